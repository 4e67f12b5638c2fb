"""Layered meshes (&MESH_DEF method='LAYERED', mesh_layers.f90) and the
element geometry of grids that are not flat (nelast 10 / 3).

The product builder and the oracle's restated setup agree bit for bit on
the reference's two layered example decks (a Q9 mesh under a SPLINE
surface with a LINEAR interface; flat layers from a file) and on a layered
mesh split by a fault; a layered mesh of flat layers runs, on the oracle's
general-geometry path, the same seismograms as the Cartesian mesh of the
same geometry on its flat path."""
import numpy as np
import pytest

from conftest import example_deck
from oracle import pyoracle as po
from sem2dpack_gb300 import Problem
from sem2dpack_gb300.deck import Layer, Material, ParDeck, Receivers, Sources, Time
from test_host_builder import assert_same_desc


def layered_box(ndof=2, curved=True, ezflt=0, ngll=5):
    from sem2dpack_gb300.distributions import Dist
    top = 1000.0
    if curved:
        top = Dist("GAUSSIAN", {"centered_at": [1000.0, 0.0], "length": [400.0, 1.0], "offset": 1000.0,
                                "ampli": 120.0}, [])
    return ParDeck(
        ngll=ngll, ndof=ndof, fmax=5.0, xlim=(0.0, 2000.0), mesh="LAYERED", zmin=0.0,
        layers=[Layer(nz=4, tag=2, ztop=400.0), Layer(nz=6, tag=1, ztop=top, quadratic=curved)],
        nelem=(16, 10), ezflt=ezflt,
        materials=[Material(tag=1, rho=2000.0, cp=3000.0, cs=1700.0),
                   Material(tag=2, rho=2400.0, cp=4200.0, cs=2400.0)],
        absorbing=[1, 2, 4],
        time=Time(kind="leapfrog", total_time=0.4, courant=0.5),
        sources=Sources(coords=[(700.0, 300.0)], f0=6.0, onset=0.2, ampli=1e9, angle=30.0),
        receivers=Receivers(number=7, first=(200.0, 900.0), last=(1800.0, 900.0), field="V", isamp=1),
    )


@pytest.mark.parametrize("name", ["TestLayers", "TestLayers_2"])
def test_example_decks_bit_exact(golden, tmp_path, name):
    dk = example_deck(golden, name, tmp_path)
    assert dk.mesh == "LAYERED"
    P, O = Problem(dk), po.OracleSetup(dk)
    a, b = P.desc(), O.desc()
    assert_same_desc(a, b)
    assert a.xjaci and a.dvol  # the reference's layered grid is never flat


@pytest.mark.parametrize("ndof,curved,ezflt", [(2, True, 0), (1, True, 0), (2, False, 5), (2, True, 5)])
def test_layered_box_bit_exact(ndof, curved, ezflt):
    dk = layered_box(ndof, curved, ezflt)
    if ezflt:
        from sem2dpack_gb300.deck import Fault
        dk.fault = Fault(tags=(5, 6), friction="SWF", values={"Tn": -100e6, "Tt": 55e6, "swf_mus": 0.6,
                                                             "swf_mud": 0.5, "swf_dc": 0.4})
        dk.sources = None
    P, O = Problem(dk), po.OracleSetup(dk)
    a, b = P.desc(), O.desc()
    assert_same_desc(a, b)
    assert a.nflt == (a.ngll - 1) * 16 + 1 if ezflt else a.nflt == 0


def test_flat_layers_equal_the_cartesian_mesh():
    """Rectangular elements: the general coefficients have zero cross terms,
    so the general path reproduces the flat one (NGLL 6: the reference's
    KD1 form on both sides)."""
    lay = layered_box(2, curved=False, ngll=6)
    lay.layers = [Layer(nz=10, tag=1, ztop=1000.0)]
    lay.materials = lay.materials[:1]
    cart = ParDeck(**{k: getattr(lay, k) for k in ("ngll", "ndof", "fmax", "xlim", "materials", "absorbing",
                                                      "time", "sources", "receivers")})
    cart.zlim, cart.nelem = (0.0, 1000.0), (16, 10)
    out = []
    for dk in (lay, cart):
        P = Problem(dk)
        d = P.desc()
        o = po.OracleSim(d, owner=P)
        o.run(200)
        out.append(o.seismograms())
    assert bool(Problem(lay).desc().xjaci) and not bool(Problem(cart).desc().xjaci)
    ref = np.linalg.norm(out[1])
    assert ref > 0 and np.linalg.norm(out[0] - out[1]) / ref <= 1e-11

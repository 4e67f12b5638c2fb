"""Strain and stress outputs on the GPU (sem2d_gpu_get_strain_stress)
against the oracle after a run: FP64 <= 1e-10 relative L2, mixed <= 1e-4;
element, node and per-point (VTI) material layouts."""
import numpy as np
import pytest

import decks
from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, Problem, Solver, workloads

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


CASES = {
    "plain_psv": lambda: workloads.plain_psv(scale=0.2, nsteps=150),
    "sh_rupture": lambda: workloads.sh_rupture(scale=0.1, nsteps=150),
    "psv_rsf": lambda: workloads.psv_rsf(scale=0.05, nsteps=150),
    "anisotropic": lambda: decks.anisotropic(),
    "kelvin_voigt": lambda: _kv(),
}


def _kv():
    """Kelvin-Voigt material: the stress is that of d + eta v (MAT_stress_dv,
    mat_gen.f90:626-641), the strain that of d."""
    dk = workloads.plain_psv(scale=0.2, nsteps=150)
    dk.materials[0].kv_eta = 0.3
    return dk


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_strain_stress_match_oracle(name, precision):
    case = CASES[name]()
    P = workloads.build(case) if name != "anisotropic" else Problem(case)
    d = P.desc()
    d.precision = precision
    g = Solver(d, owner=P)
    g.step(150)
    o = po.OracleSim(d, owner=P)
    o.run(150)
    eg, sg = g.strain_stress()
    eo, so = o.strain_stress()
    assert eg.shape == eo.shape == (d.ngll, d.ngll, d.ndof + 1, d.nelem)
    assert np.abs(so).max() > 0
    tol = 1e-10 if precision == PRECISION_FP64 else 1e-4
    assert rel_l2(eg, eo) <= tol
    assert rel_l2(sg, so) <= tol
    if name == "kelvin_voigt":  # the viscous part is present
        m = case.materials[0]
        mu = m.rho * m.cs ** 2
        assert rel_l2(sg[:, :, 2, :], 2 * mu * eo[:, :, 2, :]) > 1e-3

"""Strain and stress outputs of the oracle (MAT_strain_PSV/SH,
mat_gen.f90:727-774; MAT_ELAST_stress, mat_elastic.f90:804-862): a
displacement linear in x and z has the same strain at every GLL point
(the GLL derivative of a degree-1 polynomial is exact)."""
import numpy as np
import pytest

from oracle import pyoracle as po
from sem2dpack_gb300 import Grid, PRECISION_FP64, Problem, workloads


@pytest.mark.parametrize("ndof", [1, 2])
def test_linear_field_strain_and_stress(ndof):
    dk = workloads.plain_psv(scale=0.05, nsteps=10)
    dk.ndof = ndof
    P = Problem(dk)
    d = P.desc()
    d.precision = PRECISION_FP64
    o = po.OracleSim(d, owner=P)
    xz = Grid(dk).coord()  # (2, npoin)
    a, b, c, e = 1.5e-3, -0.7e-3, 0.4e-3, 2.1e-3
    if ndof == 2:
        disp = np.stack([a * xz[0] + b * xz[1], c * xz[0] + e * xz[1]], axis=1)
    else:
        disp = (a * xz[0] + b * xz[1])[:, None]
    o.set_displacement(disp)
    strain, stress = o.strain_stress()
    m = dk.materials[0]
    mu = m.rho * m.cs ** 2
    la = m.rho * m.cp ** 2 - 2 * mu
    if ndof == 2:
        ref_e = [a, e, 0.5 * (b + c)]
        ref_s = [(la + 2 * mu) * a + la * e, la * a + (la + 2 * mu) * e, mu * (b + c)]
    else:
        ref_e = [0.5 * a, 0.5 * b]
        ref_s = [mu * a, mu * b]
    for k in range(ndof + 1):
        np.testing.assert_allclose(strain[:, :, k, :], ref_e[k], rtol=1e-9, atol=1e-15)
        np.testing.assert_allclose(stress[:, :, k, :], ref_s[k], rtol=1e-9, atol=1e-3)

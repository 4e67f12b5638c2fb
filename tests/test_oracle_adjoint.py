"""The FP64 autograd reference of the gradient workflow (oracle/torch_ref.py)
against the C oracle: forward seismograms to round-off, and directional
derivatives of the misfit against central finite differences of the oracle
(no GPU)."""
import numpy as np
import pytest

import adjoint_cases as ac

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("ndof", [2, 1])
def test_torch_reference_gradient_matches_oracle_differences(ndof):
    m = ac.box(nx=6, nz=6, ndof=ndof, nsteps=90)
    rho, vp, vs = ac.smooth_model(m)
    true = ac.smooth_model(m, amp=0.08, seed=3)
    _, obs = ac.oracle_misfit(m, *true, np.zeros(1))
    J, sis, gr, gp, gs = ac.torch_misfit_grad(m, rho, vp, vs, obs)
    J_o, sis_o = ac.oracle_misfit(m, rho, vp, vs, obs)
    assert np.linalg.norm(sis - sis_o) <= 1e-12 * np.linalg.norm(sis_o)
    assert J == pytest.approx(J_o, rel=1e-12)
    for seed in range(2):
        dr, dp, ds = ac.smooth_direction(m, seed)
        if ndof == 1:
            dp = np.zeros_like(dp)
        eps = 1e-3
        Jp, _ = ac.oracle_misfit(m, rho + eps * dr, vp + eps * dp, vs + eps * ds, obs)
        Jm, _ = ac.oracle_misfit(m, rho - eps * dr, vp - eps * dp, vs - eps * ds, obs)
        fd = (Jp - Jm) / (2 * eps)
        an = np.sum(gr * dr) + np.sum(gp * dp) + np.sum(gs * ds)
        assert abs(an - fd) <= 1e-6 * abs(fd), (an, fd)

"""The GPU discrete adjoint (sem2d_gpu_checkpoint_every + sem2d_gpu_adjoint)
against the FP64 autograd-through-time reference (oracle/torch_ref.py,
itself pinned by finite differences of the C oracle) and against central
finite differences of the GPU FP64 forward.

Tolerances: FP64 path <= 1e-8 relative L2 on each gradient and 1e-6 on
directional derivatives; mixed path (FP32 fields, FP32 adjoint with FP64
segment sums) <= 1e-3 relative L2."""
import numpy as np
import pytest

import adjoint_cases as ac
from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, Sem2dError, Solver, workloads
from sem2dpack_gb300.gradient import forward_and_gradient

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def case(ndof, nsteps=150, nx=10):
    m = ac.box(nx=nx, nz=nx, ndof=ndof, nsteps=nsteps)
    start = ac.smooth_model(m)
    true = ac.smooth_model(m, amp=0.08, seed=3)
    J, obs, *_ = forward_and_gradient(m, *true, checkpoint_every=16)
    return m, start, obs


@pytest.mark.parametrize("ndof", [2, 1])
@pytest.mark.parametrize("every", [16, 40])
def test_adjoint_fp64_matches_autograd(ndof, every):
    m, start, obs = case(ndof)
    J, sis, gr, gp, gs = forward_and_gradient(m, *start, obs=obs, checkpoint_every=every)
    Jt, sist, tr, tp, ts = ac.torch_misfit_grad(m, *start, obs)
    assert J == pytest.approx(Jt, rel=1e-10)
    assert rel(gr, tr) <= 1e-8
    assert rel(gs, ts) <= 1e-8
    if ndof == 2:
        assert rel(gp, tp) <= 1e-8
    else:
        assert np.all(gp == 0)


def test_adjoint_fp64_matches_finite_differences():
    m, start, obs = case(2, nsteps=120)
    J, sis, gr, gp, gs = forward_and_gradient(m, *start, obs=obs, checkpoint_every=16)
    for seed in range(3):
        dr, dp, ds = ac.smooth_direction(m, seed)
        eps = 1e-3
        Jp = forward_and_gradient(m, start[0] + eps * dr, start[1] + eps * dp, start[2] + eps * ds,
                                  obs=obs, checkpoint_every=16)[0]
        Jm = forward_and_gradient(m, start[0] - eps * dr, start[1] - eps * dp, start[2] - eps * ds,
                                  obs=obs, checkpoint_every=16)[0]
        fd = (Jp - Jm) / (2 * eps)
        an = np.sum(gr * dr) + np.sum(gp * dp) + np.sum(gs * ds)
        assert abs(an - fd) <= 1e-6 * abs(fd), (seed, an, fd)


def test_adjoint_mixed_precision():
    m, start, obs = case(2)
    J, sis, gr, gp, gs = forward_and_gradient(m, *start, obs=obs, checkpoint_every=16,
                                              precision=PRECISION_MIXED)
    Jt, sist, tr, tp, ts = ac.torch_misfit_grad(m, *start, obs)
    assert J == pytest.approx(Jt, rel=1e-4)
    for g, t in ((gr, tr), (gp, tp), (gs, ts)):
        assert rel(g, t) <= 1e-3


def test_autograd_function_backward_is_the_adjoint():
    from sem2dpack_gb300.gradient import SeismogramFunction
    m, start, obs = case(2, nsteps=100)
    T = lambda a: torch.tensor(a, dtype=torch.float64, requires_grad=True)
    r, p, s = T(start[0]), T(start[1]), T(start[2])
    sis = SeismogramFunction.apply(r, p, s, m, 16)
    loss = 0.5 * torch.sum((sis - torch.tensor(obs[: sis.shape[0]])) ** 2)
    loss.backward()
    J, _, gr, gp, gs = forward_and_gradient(m, *start, obs=obs[: sis.shape[0]], checkpoint_every=16)
    assert float(loss) == pytest.approx(J, rel=1e-12)
    assert np.array_equal(r.grad.numpy(), gr) and np.array_equal(s.grad.numpy(), gs)


def test_adjoint_preconditions():
    m, start, obs = case(2, nsteps=40)
    P = workloads.build(m.deck_for(*start))
    d = P.desc()
    g = Solver(d, owner=P)  # not created for the gradient workflow
    from sem2dpack_gb300._lib import lib
    with pytest.raises(Sem2dError):
        g._check(lib().sem2d_gpu_checkpoint_every(g.h, 8))
    d.adjoint = 1
    h = Solver(d, owner=P)
    h._check(lib().sem2d_gpu_checkpoint_every(h.h, 8))
    h.step(20)  # not all steps
    res = np.zeros(d.rec_nsamp * d.nrec * d.ndof)
    pp = lambda a: a.ctypes.data_as(__import__("ctypes").POINTER(__import__("ctypes").c_double))
    with pytest.raises(Sem2dError):
        h._check(lib().sem2d_gpu_adjoint(h.h, pp(res), None, None, None))


def test_adjoint_twenty_directions():
    """Central finite differences of the FP64 forward along 20 seeded smooth
    directions."""
    m, start, obs = case(2, nsteps=100, nx=8)
    J, sis, gr, gp, gs = forward_and_gradient(m, *start, obs=obs, checkpoint_every=10)
    worst = 0.0
    for seed in range(20):
        dr, dp, ds = ac.smooth_direction(m, seed)
        eps = 1e-3
        Jp = forward_and_gradient(m, start[0] + eps * dr, start[1] + eps * dp, start[2] + eps * ds,
                                  obs=obs, checkpoint_every=10)[0]
        Jm = forward_and_gradient(m, start[0] - eps * dr, start[1] - eps * dp, start[2] - eps * ds,
                                  obs=obs, checkpoint_every=10)[0]
        fd = (Jp - Jm) / (2 * eps)
        an = np.sum(gr * dr) + np.sum(gp * dp) + np.sum(gs * ds)
        worst = max(worst, abs(an - fd) / abs(fd))
    assert worst <= 1e-6, worst


def test_adjoint_32x32_matches_autograd():
    """The FP64 autograd-through-time reference on a 32 x 32 element copy."""
    m, start, obs = case(2, nsteps=120, nx=32)
    J, sis, gr, gp, gs = forward_and_gradient(m, *start, obs=obs, checkpoint_every=24)
    Jt, sist, tr, tp, ts = ac.torch_misfit_grad(m, *start, obs)
    assert J == pytest.approx(Jt, rel=1e-10)
    for g, t in ((gr, tr), (gp, tp), (gs, ts)):
        assert rel(g, t) <= 1e-8


@pytest.mark.parametrize("ndof", [1, 2])
def test_adjoint_march_matches_strip_kernels(ndof, monkeypatch):
    """FP32: the march passes (one element per thread) against the strip
    adjoint kernel, and both against the FP64 autograd reference."""
    m, start, obs = case(ndof)
    J1, s1, *g1 = forward_and_gradient(m, *start, obs=obs, checkpoint_every=16, precision=PRECISION_MIXED)
    monkeypatch.setenv("SEM2D_MARCH", "0")
    J2, s2, *g2 = forward_and_gradient(m, *start, obs=obs, checkpoint_every=16, precision=PRECISION_MIXED)
    monkeypatch.delenv("SEM2D_MARCH")
    assert J1 == pytest.approx(J2, rel=1e-5)
    Jt, sist, *gt = ac.torch_misfit_grad(m, *start, obs)
    for a, b, t in zip(g1, g2, gt):
        if ndof == 1 and not np.any(t):
            continue  # SH has no vp gradient
        assert rel(a, b) <= 1e-4
        assert rel(a, t) <= 1e-3

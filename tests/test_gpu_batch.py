"""Batched independent problems (sem2d_gpu_create_batch) against the FP64
oracle run problem by problem, and against the single-problem GPU path.

Uneven shots of the batched-shot configuration (layered media, one
Ricker force each) at reduced size; FP64 <= 1e-10, mixed <= 1e-4 relative L2
per problem; the batched and single-problem GPU runs of a problem are
bitwise identical (same per-node summation order, same chunk height)."""
import numpy as np
import pytest
from conftest import watch_launches

from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, BatchSolver, Sem2dError, Solver, workloads

pytestmark = pytest.mark.gpu

TOL = {PRECISION_FP64: 1e-10, PRECISION_MIXED: 1e-4}


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def problems(n, precision, nsteps=200, scale=0.06):
    decks = workloads.batch_shots(nsim=n, scale=scale, nsteps=nsteps, precision=precision)
    out = []
    for dk in decks:
        P = workloads.build(dk)
        d = P.desc()
        d.precision = precision
        out.append((P, d))
    return out


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_batch_matches_oracle_per_problem(precision):
    probs = problems(5, precision)
    b = BatchSolver([d for _, d in probs], owners=[P for P, _ in probs])
    assert len(b) == 5
    b.step(200)
    assert b.current_step == 200
    sizes = set()
    for i, (P, d) in enumerate(probs):
        o = po.OracleSim(d, owner=P)
        o.run(200)
        s_o = o.seismograms()
        assert np.abs(s_o).max() > 0
        assert rel_l2(b[i].seismograms(), s_o) <= TOL[precision], i
        dg, vg = b[i].fields()
        do, vo, _ = o.fields()
        assert rel_l2(vg, vo) <= TOL[precision], i
        sizes.add(d.npoin)
    assert len(sizes) > 1  # uneven meshes


def test_batch_equals_single_problem_runs(monkeypatch):
    probs = problems(3, PRECISION_MIXED, nsteps=150)
    b = BatchSolver([d for _, d in probs], owners=[P for P, _ in probs])
    b.step(150)
    # one launch per step for the whole batch
    assert b.launches == 150 + watch_launches(150, members=3)
    monkeypatch.setenv("SEM2D_CHUNK", "16")  # the batch members' chunk height
    for i, (P, d) in enumerate(probs):
        g = Solver(d, owner=P)
        g.step(150)
        assert np.array_equal(g.seismograms(), b[i].seismograms()), i


def test_batch_reset_and_errors():
    probs = problems(2, PRECISION_FP64, nsteps=60)
    b = BatchSolver([d for _, d in probs], owners=[P for P, _ in probs])
    b.step(60)
    s0 = b[1].seismograms().copy()
    b.reset()
    assert b.current_step == 0
    b.step(60)
    assert np.array_equal(s0, b[1].seismograms())
    with pytest.raises(Sem2dError):
        b[0].step(1)  # members are stepped through their batch
    with pytest.raises(Sem2dError):
        b.step(1)  # beyond nt
    # members must agree on the number of steps
    p2 = problems(2, PRECISION_FP64, nsteps=60)
    p2[1][1].nt = 50
    with pytest.raises(Sem2dError):
        BatchSolver([d for _, d in p2], owners=[P for P, _ in p2])


def test_members_set_up_on_host_threads_equal_one_at_a_time(monkeypatch):
    """sem2d_gpu_create_batch and batch_add_many set members up on several
    host threads; the batch they build steps bit for bit like one built a
    member at a time on one thread, in the order given.  A bad member in a
    group is named and no member of that group joins the batch."""
    probs = problems(6, PRECISION_MIXED, nsteps=80)
    a = BatchSolver([d for _, d in probs], owners=[P for P, _ in probs])
    monkeypatch.setenv("SEM2D_HOST_THREADS", "1")
    b = BatchSolver(iter([d for _, d in probs]), owners=[P for P, _ in probs], group=1)
    monkeypatch.setenv("SEM2D_HOST_THREADS", "4")
    c = BatchSolver(iter([d for _, d in probs]), owners=[P for P, _ in probs], group=4)
    for s in (a, b, c):
        s.step(80)
    for i, (_, d) in enumerate(probs):
        assert a[i].desc.npoin == d.npoin
        assert np.array_equal(a[i].seismograms(), b[i].seismograms()), i
        assert np.array_equal(c[i].seismograms(), b[i].seismograms()), i
    bad = problems(3, PRECISION_MIXED, nsteps=80)
    bad[2][1].ndof = 3
    with pytest.raises(Sem2dError, match="problem 2"):
        BatchSolver([d for _, d in bad], owners=[P for P, _ in bad])

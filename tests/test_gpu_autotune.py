"""The launch-shape autotuner of the march kernels on the device: the first
handle of a class times the candidates on the first steps of its first run
and records the fastest in the tuning cache, a later handle reads it, and
the tuned run gives the same bits as the analytic shape (single problems
and batches)."""
import json

import numpy as np
import pytest

from sem2dpack_gb300 import PRECISION_MIXED, BatchSolver, Solver, workloads

pytestmark = pytest.mark.gpu

MARCH_TX = 31


def plain(scale, nsteps=100):
    P = workloads.build(workloads.plain_psv(scale=scale, nsteps=nsteps))
    d = P.desc()
    d.precision = PRECISION_MIXED
    return P, d


def test_single_problem_tuned_then_cached(monkeypatch, tmp_path):
    cache = tmp_path / "tune.json"
    monkeypatch.setenv("SEM2D_TUNE_CACHE", str(cache))
    P, d = plain(0.5)
    g = Solver(d, owner=P)
    assert g.tile[0] == MARCH_TX
    assert not cache.exists()  # timed on the first run
    g.step(100)
    assert cache.exists()
    recs = [json.loads(x) for x in cache.read_text().splitlines()]
    assert len(recs) == 1 and recs[0]["key"].startswith("march ndof=2 ")
    assert recs[0]["ms_per_step"] > 0
    launches = g.launches
    # the analytic shape gives the same bits
    monkeypatch.setenv("SEM2D_AUTOTUNE", "0")
    h = Solver(d, owner=P)
    h.step(100)
    assert np.array_equal(g.seismograms(), h.seismograms())
    assert launches == h.launches  # the timed steps are steps of the run
    monkeypatch.delenv("SEM2D_AUTOTUNE")
    # a later handle reads the cache: an entry edited by hand is taken as is
    recs[0].update(chunk_rows=3, warps_per_cta=1)
    cache.write_text(json.dumps(recs[0]) + "\n")
    k = Solver(d, owner=P)
    assert k.tile == (MARCH_TX, 3)
    k.step(100)
    assert np.array_equal(g.seismograms(), k.seismograms())


def test_batch_tuned_and_bitwise_equal(monkeypatch, tmp_path):
    cache = tmp_path / "tune.json"
    monkeypatch.setenv("SEM2D_TUNE_CACHE", str(cache))
    decks = workloads.batch_shots(nsim=4, scale=0.12, nsteps=120)
    b = BatchSolver(decks)
    b.step(120)
    recs = [json.loads(x) for x in cache.read_text().splitlines()]
    assert any("members=2^2" in r["key"] for r in recs)
    monkeypatch.setenv("SEM2D_AUTOTUNE", "0")
    c = BatchSolver(workloads.batch_shots(nsim=4, scale=0.12, nsteps=120))
    c.step(120)
    for i in range(4):
        assert np.array_equal(b[i].seismograms(), c[i].seismograms()), i

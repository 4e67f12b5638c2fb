"""Rupture time from the slip-rate series (outputs.rupture_time) against the
oracle's restatement of the reference's post-processing loop
(POST/python/post-process-fault.py:53-62), edge cases included."""
import numpy as np

from oracle import pyoracle as po
from sem2dpack_gb300.outputs import rupture_time


def test_rupture_time_matches_the_reference_loop():
    rng = np.random.default_rng(7)
    nt, nx, dt = 200, 64, 0.01
    v = np.zeros((nt, nx))
    onset = rng.integers(-5, nt + 5, size=nx)
    for x in range(nx):
        if 0 <= onset[x] < nt:
            v[onset[x]:, x] = rng.uniform(1e-3, 3.0)
    v[:, 0] = 0.5            # above the threshold from the start: no crossing
    v[:, 1] = 1e-3 * (np.arange(nt) >= 1)   # crosses exactly at the threshold
    v[:, 2] = 0.0
    v[nt - 1:, 2] = 1.0      # crosses at the last pair: outside the loop
    v[:, 3] = 0.0            # never slips
    v[:, 4] = np.where(np.arange(nt) % 20 < 10, 0.0, 2.0)  # repeated crossings: the first counts
    t, idx = rupture_time(v.T, dt)
    ref = po.rupture_time(v, dt)
    assert np.array_equal(t, ref)
    assert idx[0] == -1 and idx[2] == -1 and idx[3] == -1
    assert idx[1] == 0 and t[1] == 0.0
    assert idx[4] == 9


def test_rupture_time_short_series():
    t, idx = rupture_time(np.ones((3, 2)), 0.1)
    assert np.all(t == 0) and np.all(idx == -1)

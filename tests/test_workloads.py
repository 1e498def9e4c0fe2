"""The seeded workload generators of the batched and served configurations:
shapes, ranges and determinism (host logic, no GPU)."""
import numpy as np

from rasterjoin import synth, workloads


def test_star_set_shapes():
    rng = np.random.default_rng(5)
    xy, pidx = workloads.star_set(rng, 30, 8, 300, 200.0, 10000.0)
    assert xy.dtype == np.float32 and xy.shape[1] == 2
    assert pidx[0] == 0 and pidx[-1] == len(xy) and len(pidx) == 31
    assert np.all(np.diff(pidx) >= 3)
    assert xy.min() >= 0.0 and xy.max() <= synth.BOX


def test_served_requests_ranges_and_seed():
    a = workloads.served_requests(200, 500.0, seed=7)
    b = workloads.served_requests(200, 500.0, seed=7)
    arr = np.array([r[0] for r in a])
    assert np.all(np.diff(arr) > 0)
    assert abs(len(arr) / arr[-1] - 500.0) < 150.0          # Poisson arrivals near the offered rate
    for (t, xy, pidx, cell, (t0, t1)), other in zip(a, b):
        assert 1 <= len(pidx) - 1 <= 50
        assert cell in (1.0, 10.0, 100.0, 1000.0)
        assert synth.T0 <= t0 <= t1 <= synth.T0 + synth.YEAR
        assert workloads.HOUR <= t1 - t0 <= 30 * workloads.DAY + 1
        np.testing.assert_array_equal(xy, other[1])


def test_batched_queries_ranges():
    qs = workloads.batched_queries(24, 1_000_000_000, seed=3)
    assert len(qs) == 24
    for i, (xy, pidx, cell, (t0, t1), avg) in enumerate(qs):
        assert 1 <= len(pidx) - 1 <= 5000
        assert 1.0 <= cell <= 1000.0
        assert t0 <= t1
        assert avg == bool(i % 2)
        assert len(xy) <= 600_000 + 4 * (len(pidx) - 1)

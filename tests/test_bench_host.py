"""CPU checks of bench.py's host-side workload construction."""
import numpy as np

import bench


def test_workload_follows_requested_size(monkeypatch):
    monkeypatch.setattr(bench, "N", 4096)
    x, y, r, s = bench.make_workload()
    assert x.size == y.size == r.size == s.size == 4096
    assert abs(float(s.astype(np.float64).sum()) - 1.0) < 1e-5
    assert np.all(r == bench.SIGMA)


def test_workload_is_seeded():
    a = bench.make_workload(7, 1000)
    b = bench.make_workload(7, 1000)
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)

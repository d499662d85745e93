"""The seeded generator of batch workloads (host side, no GPU): sizes,
densities and temperatures in range, molecules inside their box with no
overlapping pair, zero net momentum, reproducible from the seed."""
import numpy as np

from ls1gb300 import batch


def test_random_boxes_ranges_and_reproducibility():
    bx = batch.random_boxes(64, 500, 20000, seed=11)
    again = batch.random_boxes(64, 500, 20000, seed=11)
    n = np.array([b.n for b in bx])
    assert n.min() >= 500 and n.max() <= 20000
    for b, c in zip(bx, again):
        assert np.array_equal(b.r, c.r) and np.array_equal(b.v, c.v)
        assert 0.05 <= b.rho <= 0.85 and 0.7 <= b.T <= 1.3
        assert np.all(b.r >= 0) and np.all(b.r < b.L)
        assert abs(b.n / np.prod(b.L) - b.rho) < 1e-9 * b.rho
        assert np.abs(b.v.sum(0)).max() < 1e-9 * b.n


def test_no_overlaps_in_the_densest_small_box():
    bx = batch.random_boxes(64, 500, 2000, rho_range=(0.80, 0.85), seed=5)
    b = min(bx, key=lambda b: b.n)
    d = b.r[:, None, :] - b.r[None, :, :]
    d -= b.L * np.round(d / b.L)
    r = np.sqrt((d ** 2).sum(-1))
    np.fill_diagonal(r, np.inf)
    assert r.min() > 0.9


def test_log_uniform_sizes():
    bx = batch.random_boxes(512, 500, 20000, seed=2024)
    ln = np.log([b.n for b in bx])
    # log-uniform on [ln 500, ln 20000]: mean of ln N near the midpoint
    assert abs(ln.mean() - 0.5 * (np.log(500) + np.log(20000))) < 0.15

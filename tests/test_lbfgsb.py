"""The hot-pixel normal-CDF fit's L-BFGS-B loop (hostmath._setulb_loop)
against scipy.optimize.minimize(method='L-BFGS-B') on the same objective:
the same points, bit for bit, on seeded histograms like the ones the
hot-pixel filter fits (zorro.py:2535-2556)."""
import numpy as np
import pytest
import scipy.optimize
import scipy.special

from zorro_gb300 import hostmath as hm


def _problem(rng, mean, size, hot):
    vals = rng.poisson(mean, size=size).astype(np.float32)
    if hot:
        vals[rng.integers(0, size, hot)] = mean * 50
    sm, ps, edges = hm.hotpix_bins(vals.mean(), 7.0)
    hist, _ = np.histogram(vals, bins=edges)
    counts = np.asarray(edges[:-1], dtype=np.float64).copy()
    counts += 0.5 * (counts[1] - counts[0])
    cdf = np.cumsum(hist.astype(np.float64))
    cdf /= cdf[-1]

    def rows(P):
        z = (counts[None, :] - P[:, 0:1]) / P[:, 1:2]
        return np.sum(np.abs(cdf[None, :] - scipy.special.ndtr(z)), axis=1)

    bounds = ((sm - 0.5 * ps, sm + 0.5 * ps), (0.7 * ps, 1.3 * ps))
    return hm._value_and_gradient(rows, bounds), (sm, ps), bounds


def test_setulb_loop_usable_here():
    assert hm._setulb_usable()


@pytest.mark.parametrize("seed", range(8))
def test_setulb_loop_matches_scipy_minimize(seed):
    rng = np.random.default_rng(100 + seed)
    for k in range(6):
        fg, x0, bounds = _problem(rng, rng.uniform(1.5, 80.0), int(rng.integers(5000, 300000)),
                                  int(rng.integers(0, 40)) if k % 2 else 0)
        ref = scipy.optimize.minimize(fg, x0, method="L-BFGS-B", bounds=bounds, jac=True).x
        got = hm._setulb_loop(fg, x0, bounds)
        assert np.array_equal(got, ref), (seed, k, got, ref)


def test_start_outside_the_bounds_is_clipped_as_scipy_does():
    rng = np.random.default_rng(7)
    fg, (sm, ps), bounds = _problem(rng, 20.0, 100000, 0)
    x0 = (sm + 3 * ps, 0.1 * ps)
    ref = scipy.optimize.minimize(fg, x0, method="L-BFGS-B", bounds=bounds, jac=True).x
    assert np.array_equal(hm._setulb_loop(fg, x0, bounds), ref)


def test_hotpix_fit_same_with_and_without_the_loop(monkeypatch):
    rng = np.random.default_rng(11)
    vals = rng.poisson(12.0, size=400000).astype(np.float32)
    vals[rng.integers(0, vals.size, 40)] = 600.0
    sm, ps, edges = hm.hotpix_bins(vals.mean(), 7.0)
    hist, _ = np.histogram(vals, bins=edges)
    info = {"cutoffLower": -4.0, "cutoffUpper": 3.25}
    monkeypatch.setattr(hm, "_SETULB_OK", True)
    a = hm.hotpix_fit(hist, edges, sm, ps, info)
    monkeypatch.setattr(hm, "_SETULB_OK", False)
    b = hm.hotpix_fit(hist, edges, sm, ps, info)
    assert a[0] == b[0] and a[1] == b[1] and a[2] == b[2] and a[3] == b[3] and a[4] == b[4]

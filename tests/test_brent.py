"""The host's bounded Brent search (hostmath.brent_bounded, used in lock step
for the preShift planes) against scipy.optimize.minimize_scalar(
method='bounded'), the optimiser of locatePeak (zorro.py:1117): the same
abscissa and the same number of function values."""
import numpy as np
import scipy.optimize

from zorro_gb300 import hostmath as hm


def _run(f, lo=0.0, hi=7.0, xatol=0.01, maxfun=15):
    g = hm.brent_bounded(lo, hi, xatol, maxfun)
    x = next(g)
    try:
        while True:
            x = g.send(f(x))
    except StopIteration as stop:
        return stop.value


def test_brent_matches_scipy_bounded():
    rng = np.random.default_rng(0)
    for _ in range(200):
        a, b, c = rng.uniform(0.5, 6.5), rng.uniform(0.1, 3.0), rng.uniform(0.0, 0.3)

        def f(x):
            return (x - a) ** 2 * b + c * np.sin(7 * x)
        res = scipy.optimize.minimize_scalar(f, bounds=[0, 7], method="bounded",
                                             options={"maxiter": 15, "xatol": 0.01})
        xb, n = _run(f)
        assert xb == res.x and n == res.nfev


def test_gaussian_taps():
    t, r = hm.gaussian_taps(0.0)
    assert r == 0 and t.tolist() == [1.0]
    t, r = hm.gaussian_taps(1.37)
    assert r == int(4 * 1.37 + 0.5) and abs(float(t.sum()) - 1.0) < 1e-6 and t[r] == t.max()

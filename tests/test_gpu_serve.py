"""Continuous batching: every movie's result is the same alone and when it
shares the GPU with others; a failing request leaves the others intact."""
import numpy as np
import pytest

from zorro_gb300.synthetic import make_movie

pytestmark = pytest.mark.gpu

DOSE = [1.0, 0.24499, -1.6649, 2.8141, 32, 0]
MIX = [
    (dict(n_frames=10, shape=(250, 240), seed=31, mean_dose=1.5, drift_sigma=0.8),
     dict(triMode="tri", shapePadded=[256, 256], fouCrop=[128, 128], maxShift=20, pixelsize=0.1,
          filterMode="dose", doseFiltParam=DOSE)),
    (dict(n_frames=12, shape=(500, 480), seed=32, mean_dose=1.0, drift_sigma=1.0, dtype="uint8", gain_map=True,
          hot_fraction=1e-3),
     dict(triMode="tri", shapePadded=[512, 512], fouCrop=[256, 256], maxShift=24, pixelsize=0.105,
          filterMode="hot,dose", doseFiltParam=DOSE)),
    (dict(n_frames=8, shape=(800, 800), seed=33, mean_dose=1.0, drift_sigma=1.2),
     dict(triMode="diag", diagWidth=3, shapePadded=[1024, 1024], fouCrop=[512, 512], maxShift=30, pixelsize=0.1)),
]


def _reg(mk, attrs, movie):
    from zorro_gb300.registrator import ImageRegistrator
    r = ImageRegistrator()
    for k, v in attrs.items():
        setattr(r, k, v)
    if mk.get("dtype") == "uint8":
        r.images, r.gainRef = movie["raw"], movie["gain"]
    else:
        r.images = movie["images"].copy()
    return r


def _compare(a, b):
    assert np.abs(a.translations - b.translations).max() <= 1e-9
    assert np.linalg.norm(a.imageSum - b.imageSum) / np.linalg.norm(b.imageSum) <= 1e-6
    if a.FRC is not None and not np.all(np.isnan(b.FRC)):
        assert np.nanmax(np.abs(a.FRC - b.FRC)) <= 1e-6
    if b.filtSum is not None:
        assert np.linalg.norm(a.filtSum - b.filtSum) / np.linalg.norm(b.filtSum) <= 1e-6


def test_alone_and_in_the_mix():
    from zorro_gb300.serve import MovieServer
    movies = [make_movie(**mk) for mk, _ in MIX]
    alone = []
    for (mk, attrs), mv in zip(MIX, movies):
        r = _reg(mk, attrs, mv)
        r.alignImageStack()
        alone.append(r)
    srv = MovieServer(slots=3, hbm_budget=40e9)
    try:
        order = [0, 1, 2, 1, 0, 2, 2, 1, 0]
        futs = [(i, srv.submit(_reg(MIX[i][0], MIX[i][1], movies[i]))) for i in order]
        for i, f in futs:
            _compare(f.result(timeout=600), alone[i])
        st = srv.stats()
        assert st["movies"] == len(order) and st["p99_s"] >= st["p50_s"] > 0
    finally:
        srv.close()


def test_failing_request_is_isolated():
    from zorro_gb300.serve import MovieServer
    mk, attrs = MIX[0]
    mv = make_movie(**mk)
    good = _reg(mk, attrs, mv)
    bad = _reg(mk, dict(attrs, shapePadded=[128, 128]), mv)  # smaller than the frames
    srv = MovieServer(slots=2)
    try:
        fb = srv.submit(bad)
        fg = srv.submit(good)
        with pytest.raises(ValueError):
            fb.result(timeout=600)
        ref = _reg(mk, attrs, mv)
        ref.alignImageStack()
        _compare(fg.result(timeout=600), ref)
    finally:
        srv.close()


def test_admission_under_a_small_budget():
    """A budget that holds one movie at a time still completes every request."""
    from zorro_gb300.serve import MovieServer, movie_bytes
    mk, attrs = MIX[0]
    mv = make_movie(**mk)
    r0 = _reg(mk, attrs, mv)
    need = movie_bytes(r0, mv["images"].shape, 4)
    srv = MovieServer(slots=3, hbm_budget=1.5 * need)
    try:
        futs = [srv.submit(_reg(mk, attrs, mv)) for _ in range(4)]
        res = [f.result(timeout=600) for f in futs]
        for r in res[1:]:
            _compare(r, res[0])
    finally:
        srv.close()


def test_even_odd_frc_alone_and_served():
    """The independent even/odd FRC runs its half-set registrations on streams
    of their own, ahead of the parent's dose filter: the same results alone
    and with two movies in flight."""
    from zorro_gb300.serve import MovieServer
    mk = dict(n_frames=24, shape=(1100, 1080), seed=41, mean_dose=1.2, drift_sigma=0.9, dtype="uint8",
              gain_map=True, hot_fraction=1e-3)
    attrs = dict(triMode="tri", shapePadded=[2048, 2048], fouCrop=[512, 512], maxShift=20, pixelsize=0.1,
                 filterMode="hot,dose", doseFiltParam=DOSE, doEvenOddFRC=True)
    mv = make_movie(**mk)
    alone = _reg(mk, attrs, mv)
    alone.alignImageStack()
    assert not np.all(np.isnan(alone.FRC))
    other = MIX[1]
    omv = make_movie(**other[0])
    srv = MovieServer(slots=2, hbm_budget=40e9)
    try:
        futs = [srv.submit(_reg(mk, attrs, mv)), srv.submit(_reg(other[0], other[1], omv)),
                srv.submit(_reg(mk, attrs, mv))]
        for f in (futs[0], futs[2]):
            r = f.result(timeout=600)
            _compare(r, alone)
            assert np.abs(np.asarray(r.transEven) - np.asarray(alone.transEven)).max() <= 1e-9
            assert np.abs(np.asarray(r.transOdd) - np.asarray(alone.transOdd)).max() <= 1e-9
            assert np.array_equal(np.isnan(np.asarray(r.FRC)), np.isnan(np.asarray(alone.FRC)))
        futs[1].result(timeout=600)
    finally:
        srv.close()

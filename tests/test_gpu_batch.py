"""Several movies registered at once (alignImageStacks, Engine.align_batch)
against each movie registered alone, and the super-resolution shape of the
batched workload against the float64 oracle.

In a batch, movies of one shape class share the launches of the forward
spectra, the frame terms, the correlation windows and the peak search; each
frame reads its own movie's gain and hot-pixel maps.  Every value is formed
by the same kernels from the same inputs as when the movie is registered
alone, so the outputs are required to be identical, not merely close.
"""
import os

import numpy as np
import pytest

from oracle import zorro_oracle as zo
from zorro_gb300.synthetic import make_movie

pytestmark = pytest.mark.gpu

DOSE = [1.0, 0.24499, -1.6649, 2.8141, 32, 0]


def make_reg(images, gain=None, **attrs):
    from zorro_gb300.registrator import ImageRegistrator
    reg = ImageRegistrator()
    reg.images = images
    reg.gainRef = gain
    for k, v in attrs.items():
        setattr(reg, k, v)
    return reg


def _movies():
    """Three movies, two shape classes, uneven frame counts: two uint8
    movies with gain maps and hot pixels (14 and 10 frames, one class; their
    half sets of 5 to 7 frames keep at least the 7 pairs the logistic weight
    fit needs) and a float32 movie of another size (10 frames)."""
    a = make_movie(14, (300, 290), seed=51, mean_dose=1.5, drift_sigma=0.9, dtype="uint8", gain_map=True,
                   hot_fraction=1e-3)
    b = make_movie(10, (300, 290), seed=52, mean_dose=1.5, drift_sigma=1.2, dtype="uint8", gain_map=True,
                   hot_fraction=1e-3)
    c = make_movie(10, (260, 250), seed=53, mean_dose=2.0, drift_sigma=0.7)
    hot = dict(triMode="tri", shapePadded=[512, 512], fouCrop=[256, 256], maxShift=20, pixelsize=0.1,
               filterMode="hot,dose", doseFiltParam=DOSE, doEvenOddFRC=True)
    plain = dict(triMode="tri", shapePadded=[512, 512], fouCrop=[256, 256], maxShift=20, pixelsize=0.1,
                 filterMode="dose", doseFiltParam=DOSE)
    return [(a["raw"], a["gain"], hot), (b["raw"], b["gain"], hot), (c["images"], None, plain)]


def _same(x, y):
    x, y = np.asarray(x), np.asarray(y)
    return x.shape == y.shape and np.array_equal(x, y, equal_nan=True)


def test_mixed_batch_equals_each_movie_alone():
    from zorro_gb300.registrator import alignImageStacks
    specs = _movies()
    alone = []
    for imgs, gain, attrs in specs:
        r = make_reg(imgs.copy(), gain, **attrs)
        r.alignImageStack()
        alone.append(r)
    batch = alignImageStacks([make_reg(imgs.copy(), gain, **attrs) for imgs, gain, attrs in specs])
    # twice: the second batch reuses the first one's buffers
    batch2 = alignImageStacks([make_reg(imgs.copy(), gain, **attrs) for imgs, gain, attrs in specs])
    for k, (r, b, b2) in enumerate(zip(alone, batch, batch2)):
        for bb in (b, b2):
            assert _same(bb.translations, r.translations), k
            assert _same(bb.errorDictList[-1]["shiftsTriMat"], r.errorDictList[-1]["shiftsTriMat"]), k
            assert _same(bb.errorDictList[-1]["peaksigTriMat"], r.errorDictList[-1]["peaksigTriMat"]), k
            assert _same(bb.imageSum, r.imageSum), k
            assert _same(bb.filtSum, r.filtSum), k
            assert _same(bb.FRC, r.FRC), k
            for key in ("guessDeadpix", "guessHotpix", "neighborPix"):
                assert bb.hotpixInfo[key] == r.hotpixInfo[key], (k, key)
            if r.doEvenOddFRC:
                assert _same(bb.transEven, r.transEven), k
                assert _same(bb.transOdd, r.transOdd), k


def test_batch_of_one_equals_alone():
    from zorro_gb300.registrator import alignImageStacks
    imgs, gain, attrs = _movies()[2]
    r = make_reg(imgs.copy(), gain, **attrs)
    r.alignImageStack()
    (b,) = alignImageStacks([make_reg(imgs.copy(), gain, **attrs)])
    assert _same(b.translations, r.translations)
    assert _same(b.imageSum, r.imageSum)


def test_superres_movie_binned_and_registered_against_oracle():
    """The super-resolution shape of the batched workload: 11520 x 8184
    counts (5 frames) Fourier-binned 2x to 5760 x 4092, padded to 6144 x 4096
    (the 6144-point transforms), cropped to 3072 x 2048, against the float64
    oracle: every pair measurement, the solve of the GPU's measurements, and
    the oracle's binned frames shifted and summed by the GPU's trajectory.
    (Ten pairs leave the logistic weight fit a single histogram bin, an
    ill-posed fit whose optimum moves with the last digits of the peak
    significances, so the trajectory is checked through the solve rather
    than against the oracle's own.)"""
    from zorro_gb300.registrator import alignImageStacks
    mv = make_movie(5, (8184, 11520), seed=61, mean_dose=1.0, drift_sigma=2.0, dtype="uint8")
    attrs = dict(triMode="tri", shapeBinned=[4092, 5760], shapePadded=[4096, 6144], fouCrop=[2048, 3072],
                 maxShift=40, pixelsize=0.05, filterMode="dose", doseFiltParam=DOSE, doLazyFRC=True)
    (reg,) = alignImageStacks([make_reg(mv["raw"], None, **attrs)])
    workers = os.cpu_count() or 1
    binned = zo.bin_stack(mv["images"], attrs["shapeBinned"], zo.Dtypes(True, workers))
    del mv
    attrs_b = {k: v for k, v in attrs.items() if k != "shapeBinned"}
    attrs_b["pixelsize"] = 0.1
    ref = zo.align_image_stack(binned, workers=workers, **attrs_b)
    assert reg.pixelsize == pytest.approx(0.1)
    ed = reg.errorDictList[-1]
    tri = ref["errorDict"]["corrTriMat"] != 0
    d = np.abs(ed["shiftsTriMat"] - ref["errorDict"]["shiftsTriMat"]).max(axis=2)[tri]
    o = zo.shifts_solver(ed["shiftsTriMat"], ed["corrTriMat"], ed["peaksigTriMat"], shapeImage=attrs["shapePadded"],
                         maxShift=attrs["maxShift"])
    t = o["translations"] - o["translations"].mean(axis=0)
    _, isum = zo.apply_shifts(binned.astype(np.float32), reg.translations, originMode=None)
    rel = np.linalg.norm(np.asarray(reg.imageSum, np.float64) - isum) / np.linalg.norm(isum)
    print("super-res: %d pairs, %d exact; solve of the GPU measurements %.2e px; imageSum rel L2 %.2e" % (
        tri.sum(), int(np.sum(d < 1e-9)), np.abs(reg.translations - t).max(), rel))
    assert np.mean(d < 1e-9) >= 0.9
    assert np.abs(reg.translations - t).max() <= 1e-6
    assert rel <= 1e-4

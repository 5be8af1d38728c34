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
ZR_EINVAL, ZR_ESIZE = -1, -3


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
    than against the oracle's own; and ten weighted equations in five
    unknowns can leave the weighted-L1 optimum a face rather than a vertex,
    so the host solve is held to the oracle's weights and objective value,
    not to the oracle solver's point of the face.)"""
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
    np.testing.assert_allclose(ed["weights"], o["weights"], rtol=1e-12)
    used = ed["corrTriMat"][:-1, 1:].astype(bool)
    A = zo.solver_matrix(used)
    f = []
    for ax in (0, 1):
        b = ed["shiftsTriMat"][:-1, 1:, ax][used]
        f.append((float(np.sum(o["weights"] * np.abs(A @ ed["relativeEst"][:, ax] - b))),
                  float(np.sum(o["weights"] * np.abs(A @ o["relativeEst"][:, ax] - b)))))
    _, isum = zo.apply_shifts(binned.astype(np.float32), reg.translations, originMode=None)
    rel = np.linalg.norm(np.asarray(reg.imageSum, np.float64) - isum) / np.linalg.norm(isum)
    print("super-res: %d pairs, %d exact; L1 objectives (GPU, oracle) %s; imageSum rel L2 %.2e" % (
        tri.sum(), int(np.sum(d < 1e-9)), f, rel))
    assert np.mean(d < 1e-9) >= 0.9
    for f_gpu, f_ora in f:
        assert abs(f_gpu - f_ora) <= 1e-9 * max(1.0, f_ora)
    assert rel <= 1e-4


def _tri(n):
    return [(i, j) for i in range(n) for j in range(i + 1, n)]


def test_batch_context_records_equal_each_movie_alone():
    """zr_ctx_create / zr_submit_batch / zr_poll / zr_wait: three movies of
    one shape (6, 9 and 5 frames) in one batch give, record for record and
    bit for bit, the peaks of each movie's own per-stage calls; a second
    batch on the same context in another order gives them again, and
    batches beyond the context's limits are refused before anything runs."""
    import ctypes as C
    import time

    import torch

    from tests import gpu_helpers as gh
    from zorro_gb300 import _lib
    P, C_, mS = (256, 256), (128, 128), 16
    movies = [make_movie(n, (200, 190), seed=70 + n, mean_dose=2.0, drift_sigma=1.0)["images"] for n in (6, 9, 5)]
    alone = []
    for imgs in movies:
        _, _, _, _, dev = gh.spectra(imgs, P, C_)
        _, _, cwin = gh.windows(dev, imgs.shape[0], C_, mS, _tri(imgs.shape[0]))
        alone.append(gh.peaks(cwin, mS))

    lib = _lib.load()
    dev = torch.cuda.current_device()
    lim = _lib.BatchLimits(200, 190, P[0], P[1], C_[0], C_[1], mS, 20, 64, 4)  # 20 frames, 61 pairs
    ctx = C.c_void_p()
    _lib.call("zr_ctx_create", dev, C.byref(lim), C.byref(ctx))
    pp = _lib.PeakParams()
    pp.sub_pix_reg, pp.bmode, pp.suppress_origin, pp.use_mask = 16, 1, 1, 1
    pp.opti_lo, pp.opti_hi, pp.opti_xatol, pp.opti_maxiter = 0.0, 7.0, 0.01, 15
    try:
        raws = [gh.dev_tensor(m.astype(np.float32)) for m in movies]
        msubs = []
        for r in raws:
            ms = torch.zeros(r.shape[0], dtype=torch.float64, device="cuda")
            _lib.call("zr_frame_sums", C.byref(gh.frames_of(r)), ms.data_ptr(), gh.stream())
            msubs.append(ms)

        def run(order):
            pairs = [np.asarray(_tri(movies[k].shape[0]), dtype=np.int32).reshape(-1) for k in order]
            outs = [np.zeros(len(p) // 2, dtype=gh.PEAK_DTYPE) for p in pairs]
            arr = (_lib.BatchMovie * len(order))()
            for slot, k in enumerate(order):
                arr[slot] = _lib.BatchMovie(gh.frames_of(raws[k]), msubs[k].data_ptr(), pairs[slot].ctypes.data,
                                            len(pairs[slot]) // 2, outs[slot].ctypes.data)
            _lib.call("zr_submit_batch", ctx, arr, len(order), C.byref(pp), gh.stream())
            t0 = time.time()
            while True:
                done = lib.zr_poll(ctx)
                assert done >= 0, _lib.last_error()
                if done == 1 or time.time() - t0 > 60:
                    break
                time.sleep(0.001)
            _lib.call("zr_wait", ctx)
            assert lib.zr_poll(ctx) == 1
            return {k: outs[slot] for slot, k in enumerate(order)}

        for order in ((0, 1, 2), (2, 0, 1)):
            got = run(order)
            for k in range(3):
                diff = [f for f in gh.PEAK_DTYPE.names
                        if got[k][f].tobytes() != alone[k][f].tobytes()]
                assert not diff, (order, k, diff, got[k][diff[0]], alone[k][diff[0]])

        # refused on the host: more frames than the context holds, a pair
        # outside its movie, a frame size of another class
        big = (_lib.BatchMovie * 3)()
        p9 = np.asarray(_tri(9), dtype=np.int32).reshape(-1)
        out9 = np.zeros(len(p9) // 2, dtype=gh.PEAK_DTYPE)
        for s in range(3):
            big[s] = _lib.BatchMovie(gh.frames_of(raws[1]), None, p9.ctypes.data, len(p9) // 2, out9.ctypes.data)
        assert lib.zr_submit_batch(ctx, big, 3, C.byref(pp), gh.stream()) == ZR_ESIZE
        bad = np.asarray([0, 9], dtype=np.int32)
        one = (_lib.BatchMovie * 1)(_lib.BatchMovie(gh.frames_of(raws[1]), None, bad.ctypes.data, 1,
                                                    out9.ctypes.data))
        assert lib.zr_submit_batch(ctx, one, 1, C.byref(pp), gh.stream()) == ZR_EINVAL
        other = gh.dev_tensor(np.zeros((4, 100, 90), np.float32))
        p4 = np.asarray(_tri(4), dtype=np.int32).reshape(-1)
        one = (_lib.BatchMovie * 1)(_lib.BatchMovie(gh.frames_of(other), None, p4.ctypes.data, len(p4) // 2,
                                                    out9.ctypes.data))
        assert lib.zr_submit_batch(ctx, one, 1, C.byref(pp), gh.stream()) == ZR_ESIZE
        torch.cuda.synchronize()
    finally:
        _lib.call("zr_ctx_destroy", ctx)

"""The whole alignImageStack on the GPU against the float64 oracle and the
reference's golden fixtures.

Tolerances (stated by the specification of this path): drift trajectory
within 0.01 px, aligned sum within 1e-4 relative L2, FRC within 1e-3
absolute, hot/dead-pixel counts exact.  Trajectories are compared after
removing the centroid, as the reference's originMode='centroid' does.
"""
import os

import numpy as np
import pytest

from oracle import zorro_oracle as zo
from zorro_gb300.synthetic import make_movie

pytestmark = pytest.mark.gpu

DOSE = [1.0, 0.24499, -1.6649, 2.8141, 32, 0]
TRAJ_TOL = 0.01
SUM_TOL = 1e-4
FRC_TOL = 1e-3


def gpu_align(images, gain=None, **attrs):
    from zorro_gb300.registrator import ImageRegistrator
    reg = ImageRegistrator()
    reg.images = images
    reg.gainRef = gain
    for k, v in attrs.items():
        setattr(reg, k, v)
    reg.alignImageStack()
    return reg


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


CASES = {
    "tri_crop_dose": (dict(n_frames=8, shape=(200, 180), seed=3, mean_dose=2.0, drift_sigma=1.0),
                      dict(triMode="tri", shapePadded=[256, 256], fouCrop=[128, 128], maxShift=20, pixelsize=0.1,
                           filterMode="dose", doseFiltParam=DOSE)),
    "diag_nocrop": (dict(n_frames=12, shape=(240, 256), seed=4, mean_dose=1.5, drift_sigma=0.7),
                    dict(triMode="diag", diagWidth=4, shapePadded=[256, 256], fouCrop=[256, 256], maxShift=24,
                         pixelsize=0.1)),
    "frc_800": (dict(n_frames=6, shape=(800, 800), seed=5, mean_dose=1.0, drift_sigma=1.2),
                dict(triMode="tri", shapePadded=[1024, 1024], fouCrop=[1024, 1024], maxShift=30, pixelsize=0.1,
                     filterMode="dose", doseFiltParam=DOSE)),
    # full triangles large enough for a well-posed logistic fit (>= 27 bins)
    "tri24_crop": (dict(n_frames=24, shape=(250, 240), seed=12, mean_dose=1.5, drift_sigma=0.8),
                   dict(triMode="tri", shapePadded=[256, 256], fouCrop=[128, 128], maxShift=20, pixelsize=0.1,
                        filterMode="dose", doseFiltParam=DOSE)),
    "tri20_frc": (dict(n_frames=20, shape=(780, 800), seed=13, mean_dose=1.0, drift_sigma=0.8),
                  dict(triMode="tri", shapePadded=[1024, 1024], fouCrop=[512, 512], maxShift=24, pixelsize=0.1,
                       filterMode="dose", doseFiltParam=DOSE)),
    # crop and padded sizes of 3 x 2^k (mixed-radix transforms)
    "tri20_crop768": (dict(n_frames=20, shape=(700, 650), seed=14, mean_dose=1.5, drift_sigma=0.8),
                      dict(triMode="tri", shapePadded=[1536, 1536], fouCrop=[768, 768], maxShift=30, pixelsize=0.1,
                           filterMode="dose", doseFiltParam=DOSE, doLazyFRC=False)),
}
WELL_POSED = ("tri24_crop", "tri20_frc", "tri20_crop768")


@pytest.fixture(scope="module", params=sorted(CASES))
def aligned_pair(request):
    mk, attrs = CASES[request.param]
    mv = make_movie(**mk)
    reg = gpu_align(mv["images"].copy(), **attrs)
    ref = zo.align_image_stack(mv["images"], **attrs)
    return request.param, mv, reg, ref


def test_pair_measurements(aligned_pair):
    """Every pair's shift, peak significance and correlation from the GPU
    kernels against the float64 oracle."""
    name, mv, reg, ref = aligned_pair
    ed, eo = reg.errorDictList[-1], ref["errorDict"]
    tri = eo["corrTriMat"] != 0
    assert np.array_equal(ed["corrTriMat"] != 0, tri)
    d = np.abs(ed["shiftsTriMat"] - eo["shiftsTriMat"]).max(axis=2)[tri]
    step = reg.shapePadded[0] / (2 * np.floor(reg.fouCrop[0] / 2)) / reg.subPixReg
    assert np.mean(d < 1e-9) >= 0.97, (name, d)
    assert d.max() <= 2 * step + 1e-9
    np.testing.assert_allclose(ed["peaksigTriMat"][tri], eo["peaksigTriMat"][tri], rtol=2e-3)
    np.testing.assert_allclose(ed["originTriMat"][tri], eo["originTriMat"][tri], rtol=1e-3,
                               atol=1e-4 * np.abs(eo["originTriMat"]).max())


def test_solver_on_gpu_measurements(aligned_pair):
    """The host solve fed the GPU's pair measurements is an exact optimum of
    the oracle's problem for them (same weights, same objective value); on
    full triangles, where the optimum is a single vertex, the same
    trajectory."""
    name, mv, reg, ref = aligned_pair
    ed = reg.errorDictList[-1]
    o = zo.shifts_solver(ed["shiftsTriMat"], ed["corrTriMat"], ed["peaksigTriMat"], shapeImage=reg.shapePadded,
                         maxShift=reg.maxShift)
    np.testing.assert_allclose(ed["weights"], o["weights"], rtol=1e-12)
    tri = ed["corrTriMat"][:-1, 1:].astype(bool)
    A = zo.solver_matrix(tri)
    w = o["weights"]
    for ax in (0, 1):
        b = ed["shiftsTriMat"][:-1, 1:, ax][tri]
        f_gpu = np.sum(w * np.abs(A @ ed["relativeEst"][:, ax] - b))
        f_ora = np.sum(w * np.abs(A @ o["relativeEst"][:, ax] - b))
        assert abs(f_gpu - f_ora) <= 1e-9 * max(1.0, f_ora), (ax, f_gpu, f_ora)
    if reg.triMode != "diag":
        t = o["translations"] - o["translations"].mean(axis=0)
        assert np.abs(reg.translations - t).max() <= 1e-6


def test_trajectory_well_posed(aligned_pair):
    """End to end within 0.01 px of the float64 oracle where the logistic
    weight fit is well posed.  With a handful of pairs the fit has 2-4
    histogram bins and its optimum drifts with 1e-7 changes of the peak
    significances; banded triangles make the weighted-L1 optimum a flat face.
    Those cases are held to the checks above instead."""
    name, mv, reg, ref = aligned_pair
    if name not in WELL_POSED:
        pytest.skip("ill-posed weight fit / degenerate L1 face: covered by the consistency checks")
    assert np.abs(reg.translations - ref["translations"]).max() <= TRAJ_TOL


def _downstream(mv, reg, attrs):
    """The oracle's shift/sum, FRC and dose filter run with the GPU's trajectory."""
    dt = zo.Dtypes(True)
    imgs = mv["images"].astype(np.float32).copy()
    _, isum = zo.apply_shifts(imgs, reg.translations, originMode=None)
    out = {"imageSum": isum}
    frc, _, _ = zo.lazy_frc(imgs, reg.translations, dt=dt)
    out["FRC"] = frc
    if attrs.get("filterMode") == "dose":
        out["filtSum"] = zo.dose_filter(imgs, attrs["shapePadded"], attrs["pixelsize"], 300.0, attrs["doseFiltParam"],
                                        isum, dt=dt)
    return out


@pytest.fixture(scope="module")
def downstream(aligned_pair):
    name, mv, reg, ref = aligned_pair
    return _downstream(mv, reg, CASES[name][1])


def test_aligned_sum(aligned_pair, downstream):
    name, mv, reg, ref = aligned_pair
    assert rel_l2(reg.imageSum, downstream["imageSum"]) <= SUM_TOL
    if name in WELL_POSED:
        assert rel_l2(reg.imageSum, ref["imageSum"]) <= SUM_TOL


def test_frc(aligned_pair, downstream):
    name, mv, reg, ref = aligned_pair
    if CASES[name][1].get("doLazyFRC") is False:
        assert reg.FRC is None and "FRC" not in ref
        return
    want = downstream["FRC"]
    if np.all(np.isnan(want)):
        assert np.all(np.isnan(reg.FRC))
        return
    assert np.nanmax(np.abs(reg.FRC - want)) <= FRC_TOL
    if name in WELL_POSED:
        assert np.nanmax(np.abs(reg.FRC - ref["FRC"])) <= FRC_TOL


def test_dose_filtered_sum(aligned_pair, downstream):
    name, mv, reg, ref = aligned_pair
    if "filtSum" not in downstream:
        pytest.skip("no dose filter in this case")
    assert rel_l2(reg.filtSum, downstream["filtSum"]) <= SUM_TOL
    if name in WELL_POSED:
        assert rel_l2(reg.filtSum, ref["filtSum"]) <= SUM_TOL


def test_hot_pixels_and_gain():
    mv = make_movie(20, (256, 240), seed=11, mean_dose=1.6, drift_sigma=0.8, dtype="uint8", gain_map=True,
                    hot_fraction=1e-3)
    attrs = dict(triMode="diag", diagWidth=3, shapePadded=[256, 256], fouCrop=[256, 256], maxShift=24,
                 pixelsize=0.105, filterMode="hot")
    reg = gpu_align(mv["raw"], gain=mv["gain"], **attrs)
    ref = zo.align_image_stack(mv["images"], **attrs)
    for k in ("guessDeadpix", "guessHotpix", "neighborPix"):
        assert reg.hotpixInfo[k] == ref["hotpixInfo"][k], k
    tri = ref["errorDict"]["corrTriMat"] != 0
    d = np.abs(reg.errorDictList[-1]["shiftsTriMat"] - ref["errorDict"]["shiftsTriMat"]).max(axis=2)[tri]
    assert np.mean(d < 1e-9) >= 0.95
    # the hot-pixel-corrected stack shifted by the GPU's own trajectory
    filt, _, _ = zo.hotpix_filter(mv["images"].copy(), dict(zo.DEFAULTS["hotpixInfo"]), dt=zo.Dtypes(True))
    _, isum = zo.apply_shifts(filt, reg.translations, originMode=None)
    assert rel_l2(reg.imageSum, isum) <= SUM_TOL


def _golden_names():
    from tests.golden.make_golden import CASES as GC
    return sorted(GC)


@pytest.mark.parametrize("name", _golden_names())
def test_golden_fixtures(name):
    """Against the unmodified reference's own outputs (tests/golden), one
    case per test so that a log names every case compared or skipped."""
    from tests.golden.make_golden import CASES as GC, input_checksum
    case = GC[name]
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz")))
    mv = make_movie(**case["movie"])
    if input_checksum(mv["images"]) != str(g["checksum"]):
        pytest.skip("%s: the synthetic input differs on this platform" % name)
    attrs = dict(case["attrs"])
    if case["movie"].get("dtype") == "uint8":
        reg = gpu_align(mv["raw"], gain=mv["gain"], **attrs)
    else:
        reg = gpu_align(mv["images"].copy(), **attrs)
    tri = g["corrTriMat"] != 0
    d = np.abs(reg.errorDictList[-1]["shiftsTriMat"] - g["shiftsTriMat"]).max(axis=2)[tri]
    assert np.mean(d < 1e-9) >= 0.95, (name, d)
    same_traj = np.abs(reg.translations - g["translations"]).max() <= TRAJ_TOL
    vals = np.asarray(reg.imageSum, np.float64).reshape(-1)[g["imageSum_idx"]]
    if same_traj:
        assert np.linalg.norm(vals - g["imageSum_val"]) / np.linalg.norm(g["imageSum_val"]) <= SUM_TOL, name
    if same_traj and "FRC" in g and not np.all(np.isnan(g["FRC"])):
        assert np.nanmax(np.abs(reg.FRC - g["FRC"])) <= FRC_TOL, name
    if "hot_guessHotpix" in g:
        # exact against the oracle on this platform; the fixture was made on
        # another NumPy/SciPy build, whose normal-CDF fit (L-BFGS-B) can
        # move a pixel sitting on the cut-off
        ref = zo.align_image_stack(mv["images"], **attrs)
        for k in ("guessDeadpix", "guessHotpix", "neighborPix"):
            assert reg.hotpixInfo[k] == ref["hotpixInfo"][k], (name, k)
            assert abs(reg.hotpixInfo[k] - int(g["hot_" + k])) <= 1 + 0.01 * int(g["hot_" + k]), (name, k)


def test_even_odd_frc_against_oracle():
    """Independent half-set FRC (doEvenOddFRC): 40 frames, so that each half
    (20 frames, 190 pairs) has a well-posed weight fit; the half-set
    trajectories within 0.01 px and the FRC within 1e-3 of the float64
    oracle."""
    mv = make_movie(n_frames=40, shape=(800, 780), seed=31, mean_dose=1.5, drift_sigma=0.8)
    attrs = dict(triMode="tri", shapePadded=[1024, 1024], fouCrop=[512, 512], maxShift=20, pixelsize=0.1,
                 doEvenOddFRC=True)
    reg = gpu_align(mv["images"].copy(), **attrs)
    ref = zo.align_image_stack(mv["images"], **attrs)
    assert np.abs(reg.translations - ref["translations"]).max() <= TRAJ_TOL
    assert np.abs(reg.transEven - ref["transEven"]).max() <= TRAJ_TOL
    assert np.abs(reg.transOdd - ref["transOdd"]).max() <= TRAJ_TOL
    assert reg.FRC.shape == ref["FRC"].shape
    assert not np.all(np.isnan(ref["FRC"]))
    assert np.nanmax(np.abs(np.asarray(reg.FRC) - ref["FRC"])) <= FRC_TOL
    assert np.array_equal(np.isnan(np.asarray(reg.FRC)), np.isnan(ref["FRC"]))


def test_fourier_shift_raises_like_the_reference():
    """shiftMethod 'fourier' stops the reference in xcorrnm2_tri
    (AttributeError, zorro.py:895); the GPU path refuses it the same way."""
    mv = make_movie(n_frames=4, shape=(120, 112), seed=2, mean_dose=2.0, drift_sigma=0.5)
    with pytest.raises(AttributeError):
        gpu_align(mv["images"].copy(), triMode="tri", shapePadded=[128, 128], fouCrop=[128, 128], maxShift=16,
                  pixelsize=0.1, shiftMethod="fourier")
    with pytest.raises(AttributeError):
        zo.align_image_stack(mv["images"], triMode="tri", shapePadded=[128, 128], fouCrop=[128, 128], maxShift=16,
                             pixelsize=0.1, shiftMethod="fourier", weightMode="autologistic")


def test_refine_mode_against_oracle():
    """triMode 'refine': every frame against the sum of the others."""
    mv = make_movie(n_frames=12, shape=(240, 256), seed=8, mean_dose=1.5, drift_sigma=0.7)
    attrs = dict(triMode="refine", shapePadded=[256, 256], fouCrop=[256, 256], maxShift=24, pixelsize=0.1)
    reg = gpu_align(mv["images"].copy(), **attrs)
    ref = zo.align_image_stack(mv["images"], **attrs)
    ed, eo = reg.errorDictList[-1], ref["errorDict"]
    d = np.abs(np.diagonal(ed["shiftsTriMat"], axis1=0, axis2=1) - np.diagonal(eo["shiftsTriMat"], axis1=0, axis2=1))
    assert np.mean(d.max(axis=0) < 1e-9) >= 0.9, d
    assert np.abs(reg.translations - ref["translations"]).max() <= 1.0 / 16 + 1e-6
    assert rel_l2(reg.imageSum, ref["imageSum"]) <= 1e-3


@pytest.mark.parametrize("name", WELL_POSED)
def test_half_precision_spectra(name):
    """spectraPrecision 'float16' (frame spectra in half precision with
    per-spectrum power-of-two scales, float32 arithmetic): the error against
    the float64 oracle, reported and bounded."""
    mk, attrs = CASES[name]
    mv = make_movie(**mk)
    reg = gpu_align(mv["images"].copy(), spectraPrecision="float16", **attrs)
    ref = zo.align_image_stack(mv["images"], **attrs)
    ed, eo = reg.errorDictList[-1], ref["errorDict"]
    tri = eo["corrTriMat"] != 0
    d = np.abs(ed["shiftsTriMat"] - eo["shiftsTriMat"]).max(axis=2)[tri]
    rmse = float(np.sqrt(np.mean((reg.translations - ref["translations"]) ** 2)))
    print("%s float16 spectra: pairs exact %.3f, trajectory rmse %.4f px, max %.4f px, sum rel L2 %.2e" % (
        name, np.mean(d < 1e-9), rmse, np.abs(reg.translations - ref["translations"]).max(),
        rel_l2(reg.imageSum, ref["imageSum"])))
    # the pair measurements stay exact but the peak significances move by
    # half-precision noise, which can tip the logistic weights and with them
    # the L1 optimum's vertex: bounds, not the 0.01 px of float32 spectra
    assert np.mean(d < 1e-9) >= 0.9
    assert rmse <= 0.05
    assert np.abs(reg.translations - ref["translations"]).max() <= 0.25
    assert rel_l2(reg.imageSum, ref["imageSum"]) <= 2e-2


def test_binned_movie_against_oracle():
    """shapeBinned: the movie Fourier-binned 2x on the GPU, then registered."""
    mv = make_movie(n_frames=20, shape=(1400, 1300), seed=23, mean_dose=0.5, drift_sigma=1.2)
    attrs = dict(triMode="tri", shapeBinned=[700, 650], shapePadded=[1024, 1024], fouCrop=[512, 512], maxShift=30,
                 pixelsize=0.05, filterMode="dose", doseFiltParam=DOSE)
    reg = gpu_align(mv["images"].copy(), **attrs)
    ref = zo.align_image_stack(mv["images"], **attrs)
    assert reg.pixelsize == pytest.approx(ref["pixelsize"])
    assert np.abs(reg.translations - ref["translations"]).max() <= TRAJ_TOL
    assert rel_l2(reg.imageSum, ref["imageSum"]) <= SUM_TOL
    assert rel_l2(reg.filtSum, ref["filtSum"]) <= SUM_TOL


@pytest.mark.parametrize("shape", [(200, 180), (201, 183)])
def test_strided_frame_selection_reads_in_place(shape):
    """Every other frame of a device stack (how the even/odd FRC hands the
    aligned halves on) registers exactly like its contiguous copy; the
    201 x 183 movie's odd-frame view starts off a 16-byte boundary and is
    copied, the 200 x 180 one is read in place through its frame stride."""
    import torch
    mv = make_movie(12, shape, seed=6, mean_dose=2.0, drift_sigma=0.8)
    dev = torch.from_numpy(mv["images"]).cuda()
    attrs = dict(triMode="tri", shapePadded=[256, 256], fouCrop=[256, 256], maxShift=16, doLazyFRC=False)
    a = gpu_align(dev[1::2], **attrs)
    b = gpu_align(dev[1::2].contiguous(), **attrs)
    assert np.array_equal(a.translations, b.translations)
    assert np.array_equal(a.imageSum, b.imageSum)


@pytest.mark.parametrize("dtype,shape", [("uint16", (300, 290)), ("float16", (301, 291)), ("uint8", (301, 291))])
def test_raw_counts_with_gain_equal_corrected_frames(dtype, shape):
    """Raw detector counts (uint8 / uint16 / float16) with gainRef give the
    same registration, bit for bit, as the float32 frames float32(gain * raw)
    (loadData's gain multiply, zorro.py:3466, fused into every frame read):
    hot-pixel counts, trajectory, sums, FRC."""
    mv = make_movie(10, shape, seed=13, mean_dose=1.5, drift_sigma=0.8, dtype="uint8", gain_map=True,
                    hot_fraction=1e-3)
    raw = mv["raw"].astype(dtype)
    gain = mv["gain"].astype(np.float32)
    frames = (gain[None, :, :] * raw.astype(np.float32)).astype(np.float32)
    attrs = dict(triMode="tri", shapePadded=[512, 512], fouCrop=[256, 256], maxShift=20, pixelsize=0.1,
                 filterMode="hot,dose", doseFiltParam=DOSE)
    a = gpu_align(raw, gain=gain, **attrs)
    b = gpu_align(frames, **attrs)
    for k in ("guessDeadpix", "guessHotpix", "neighborPix"):
        assert a.hotpixInfo[k] == b.hotpixInfo[k], k
    assert np.array_equal(a.translations, b.translations)
    assert np.array_equal(a.imageSum, b.imageSum)
    assert np.array_equal(a.filtSum, b.filtSum)
    assert np.array_equal(np.asarray(a.FRC), np.asarray(b.FRC), equal_nan=True)

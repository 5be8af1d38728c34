"""Generate the golden fixtures by running the UNMODIFIED reference.

Run from the repository root with ``ZORRO_REF_ROOT`` naming a checkout of
LBEM-CH/zorro (required; the directory that holds ``zorro/zorro.py``):

    ZORRO_REF_ROOT=<checkout> python tests/golden/make_golden.py

Each case regenerates its input movie from ``zorro_gb300.synthetic`` with a
fixed seed, runs ``ImageRegistrator.alignImageStack`` through
``oracle/ref_harness.py`` in float64 and stores the reference's outputs (and a
checksum of the input) in ``tests/golden/<case>.npz``.  Large arrays are
stored as a fixed random subset of pixels plus their total.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from zorro_gb300.synthetic import make_movie  # noqa: E402

DOSE = [1.0, 0.24499, -1.6649, 2.8141, 32, 0]

CASES = {
    # Fourier cropping (P=256 -> C=128), full triangle, dose filter
    "crop_dose": dict(movie=dict(n_frames=8, shape=(200, 180), seed=3, mean_dose=2.0, drift_sigma=1.0),
                      attrs=dict(triMode="tri", shapePadded=[256, 256], fouCrop=[128, 128], maxShift=20,
                                 pixelsize=0.1, filterMode="dose", doseFiltParam=DOSE)),
    # gain + hot pixels, banded triangle
    "hot_diag": dict(movie=dict(n_frames=20, shape=(256, 240), seed=11, mean_dose=1.6, drift_sigma=0.8,
                                dtype="uint8", gain_map=True, hot_fraction=1e-3),
                     attrs=dict(triMode="diag", diagWidth=3, shapePadded=[256, 256], fouCrop=[256, 256],
                                maxShift=24, pixelsize=0.105, filterMode="hot")),
    # large enough for tiled FRC (one 512^2 tile), no crop
    "frc_800": dict(movie=dict(n_frames=6, shape=(800, 800), seed=5, mean_dose=1.0, drift_sigma=1.2),
                    attrs=dict(triMode="tri", shapePadded=[1024, 1024], fouCrop=[1024, 1024], maxShift=30,
                               pixelsize=0.1, filterMode="dose", doseFiltParam=DOSE)),
    # independent half-set FRC: even/odd frames re-registered (with the hot-pixel
    # filter), the two sums aligned in 'first' mode, tiled FRC of the pair
    # (40 frames: each half has 190 pairs, enough for a well-posed weight fit)
    "evenodd_frc": dict(movie=dict(n_frames=40, shape=(800, 780), seed=21, mean_dose=1.5, drift_sigma=0.8),
                        attrs=dict(triMode="tri", shapePadded=[1024, 1024], fouCrop=[512, 512], maxShift=20,
                                   pixelsize=0.1, doEvenOddFRC=True)),
    # a Fourier crop of 3 x 2^k (the reference's default crop is 3072) with the dose filter
    "crop768": dict(movie=dict(n_frames=12, shape=(700, 650), seed=17, mean_dose=1.5, drift_sigma=1.0),
                    attrs=dict(triMode="diag", diagWidth=4, shapePadded=[1024, 1024], fouCrop=[768, 768],
                               maxShift=30, pixelsize=0.1, filterMode="dose", doseFiltParam=DOSE,
                               doLazyFRC=False)),
    # Fourier binning (binStack) of 1400 x 1300 frames to 700 x 650, then the usual path
    "bin_fourier": dict(movie=dict(n_frames=12, shape=(1400, 1300), seed=19, mean_dose=0.5, drift_sigma=1.5),
                        attrs=dict(triMode="tri", shapeBinned=[700, 650], shapePadded=[1024, 1024],
                                   fouCrop=[512, 512], maxShift=30, pixelsize=0.05, filterMode="dose",
                                   doseFiltParam=DOSE)),
    # refine mode: each frame against the sum of the others, no solver
    "refine_mode": dict(movie=dict(n_frames=10, shape=(200, 180), seed=12, mean_dose=1.5, drift_sigma=0.8),
                        attrs=dict(triMode="refine", shapePadded=[256, 256], fouCrop=[128, 128], maxShift=20,
                                   pixelsize=0.1, doLazyFRC=False)),
    # preShift: uncropped correlation planes, the maxShift disc rolled to the
    # previous pair of each row (a drift larger than the disc over the row)
    "preshift": dict(movie=dict(n_frames=8, shape=(120, 128), seed=23, mean_dose=3.0, drift_sigma=2.5),
                     attrs=dict(triMode="tri", shapePadded=[128, 128], fouCrop=[128, 128], maxShift=8,
                                pixelsize=0.1, preShift=True, doLazyFRC=False)),
    # auto mode: each row stops at the first weak pair or at autoMax frames
    "auto_mode": dict(movie=dict(n_frames=14, shape=(200, 180), seed=29, mean_dose=1.2, drift_sigma=0.8),
                      attrs=dict(triMode="auto", autoMax=6, peaksigThres=5.6, shapePadded=[256, 256],
                                 fouCrop=[128, 128], maxShift=20, pixelsize=0.1, doLazyFRC=False)),
    # fixed Gaussian peak filter (Bmode 'conv' from Brad), peak-significance
    # weights, 4x sub-pixel upsampling, normalised dose filter
    "conv_corr": dict(movie=dict(n_frames=10, shape=(200, 180), seed=31, mean_dose=1.5, drift_sigma=0.8),
                      attrs=dict(triMode="tri", shapePadded=[256, 256], fouCrop=[128, 128], maxShift=20,
                                 pixelsize=0.1, Bmode="conv", Brad=40, weightMode="corr", subPixReg=4,
                                 filterMode="dosenorm", doseFiltParam=DOSE, doLazyFRC=False)),
    # template mode: correlate everything to frame 0, no solver
    "first_mode": dict(movie=dict(n_frames=5, shape=(120, 128), seed=21, mean_dose=3.0, drift_sigma=1.0),
                       attrs=dict(triMode="first", shapePadded=[128, 128], fouCrop=[128, 128], maxShift=16,
                                  pixelsize=0.1, doLazyFRC=False)),
}


def input_checksum(images):
    return hashlib.sha256(np.ascontiguousarray(images, dtype=np.float32).tobytes()).hexdigest()


def subset(name, arr, out, n=4096, seed=0):
    arr = np.asarray(arr, dtype=np.float64)
    flat = arr.reshape(-1)
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(flat.size, size=min(n, flat.size), replace=False))
    out[name + "_idx"] = idx
    out[name + "_val"] = flat[idx]
    out[name + "_shape"] = np.array(arr.shape)
    out[name + "_total"] = np.array(np.sum(flat))


def main(names=None):
    from oracle import ref_harness as rh
    for name, case in CASES.items():
        if names and name not in names:
            continue
        mv = make_movie(**case["movie"])
        attrs = dict(case["attrs"])
        reg = rh.run_reference(mv["images"].copy(), capture=True, **attrs)
        ed = reg.errorDictList[-1]
        out = {"checksum": np.array(input_checksum(mv["images"]))}
        for k in ("shiftsTriMat", "corrTriMat", "peaksigTriMat", "originTriMat"):
            out[k] = np.asarray(ed[k], dtype=np.float64)
        for k in ("weights", "errorX", "errorY", "relativeEst"):
            if k in ed:
                out[k] = np.asarray(ed[k], dtype=np.float64)
        for k in ("peaksigThres", "logisticK", "logisticNu", "mean_errorNorm", "std_errorNorm"):
            if k in ed:
                out[k] = np.array(float(ed[k]))
        out["translations"] = np.asarray(reg.translations, dtype=np.float64)
        subset("imageSum", reg.imageSum, out)
        if reg.FRC is not None:
            out["FRC"] = np.asarray(reg.FRC, dtype=np.float64)
            subset("FRC2D", reg.FRC2D, out)
        if reg.filtSum is not None:
            subset("filtSum", reg.filtSum, out)
        if attrs.get("doEvenOddFRC"):
            out["transEven"] = np.asarray(reg.transEven, dtype=np.float64)
            out["transOdd"] = np.asarray(reg.transOdd, dtype=np.float64)
        if "hot" in (attrs.get("filterMode") or ""):
            for k in ("guessDeadpix", "guessHotpix", "neighborPix", "cutoffLower", "cutoffUpper",
                      "frameMean", "frameStd"):
                out["hot_" + k] = np.array(reg.hotpixInfo[k])
        pairs = sorted(reg._cap["C"])[:4]
        out["cap_pairs"] = np.array(pairs)
        for i, p in enumerate(pairs):
            out["cap_C_%d" % i] = reg._cap["C"][p]
            out["cap_Cfilt_%d" % i] = reg._cap["Cfilt"][p]
        path = os.path.join(ROOT, "tests", "golden", name + ".npz")
        np.savez_compressed(path, **out)
        print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main(sys.argv[1:])

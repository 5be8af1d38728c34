"""Generate the .zor fixtures by running the UNMODIFIED reference's
saveConfig / loadConfig (zorro/zorro.py:3682-4075) through
oracle/ref_harness.py (``ZORRO_REF_ROOT`` names the reference checkout).

    ZORRO_REF_ROOT=<checkout> python tests/golden/make_config_golden.py

Writes tests/golden/config_ref.zor (the reference's saveConfig of the state
in ``config_state()``) and tests/golden/config_ref_loaded.json (what the
reference's loadConfig sets when it reads that file into a fresh
registrator).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

LOADED_ATTRS = ["verbose", "umask", "fftw_effort", "n_threads", "saveC", "METAstatus", "cachePath", "pixelsize",
                "voltage", "C3", "gain", "detectorPixelSize", "gainInfo", "trackCorrStats", "corrStats", "bench",
                "hotpixInfo", "translations", "transEven", "transOdd", "FRC", "CTFProgram", "ctfInfo", "xcorrMode",
                "triMode", "startFrame", "endFrame", "shapePadded", "shapeOriginal", "shapeBinned", "fouCrop",
                "subPixReg", "shiftMethod", "maxShift", "preShift", "diagWidth", "diagStart", "autoMax",
                "peaksigThres", "corrThres", "velocityThres", "Brad", "Bmode", "BfiltType", "originMode",
                "suppressOrigin", "weightMode", "logisticK", "logisticNu", "filterMode", "doFRC", "doLazyFRC",
                "doEvenOddFRC", "doseFiltParam", "files", "savePNG", "compress_ext", "saveMovie", "doCompression",
                "plotDict", "errorDictList"]


def config_state():
    """A registrator state with non-default values in every section."""
    files = {"config": "config_ref.zor", "stack": "movie_001.mrc", "mask": None, "sum": "sum/movie_001_zorro.mrc",
             "align": "align/movie_001_zorro_movie.mrcs", "figurePath": "figs", "xc": None, "moveRawPath": None,
             "original": None, "gainRef": "gain.mrc", "stdout": None, "automatch": None, "rejected": None,
             "compressor": None, "clevel": 1}
    return dict(
        verbose=1, METAstatus="fini", n_threads=8, cachePath="cache", pixelsize=0.105, voltage=300.0, C3=2.7,
        gain=1.2, detectorPixelSize=5.0,
        gainInfo={"Horizontal": True, "Vertical": False, "Diagonal": True, "GammaParams": [0.12, -1.04, -0.03, 1.04]},
        xcorrMode="zorro", triMode="tri", shapePadded=[4096, 4096], shapeOriginal=[3838, 3710], shapeBinned=None,
        fouCrop=[2048, 2048], subPixReg=16, shiftMethod="lanczos", maxShift=100, preShift=False, diagStart=1,
        diagWidth=6, autoMax=12, startFrame=0, endFrame=0, peaksigThres=6.5, corrThres=None, velocityThres=None,
        Brad=512, Bmode="opti", BfiltType="gaussian", originMode="centroid", weightMode="autologistic",
        logisticK=5.5, logisticNu=0.25, suppressOrigin=True, filterMode="hot,dose", doLazyFRC=False,
        doEvenOddFRC=True, doseFiltParam=[1.2, 0.24499, -1.6649, 2.8141, 32, 0], CTFProgram=None, savePNG=False,
        compress_ext=".bz2", saveMovie=True, doCompression=False, files=files,
        translations=np.array([[0.0, 0.5], [1.25, -2.0], [3.0, 4.5]]), transEven=None, transOdd=None,
        FRC=np.array([1.0, 0.75, 0.5, 0.125]),
        hotpixInfo={"logisticK": 6.0, "relax": 0.925, "maxSigma": 8.0, "psf": "K2", "guessHotpix": 12,
                    "guessDeadpix": 3, "decorrOutliers": False, "cutoffLower": -4.0, "cutoffUpper": 3.5,
                    "neighborPix": 40},
        trackCorrStats=False, corrStats=None, bench={"align0": 1.5, "align1": 2.25},
        errorDictList=[{"shiftsTriMat": np.arange(18, dtype=float).reshape(3, 3, 2) / 16.0, "M": 3,
                        "mean_errorNorm": 0.125, "relativeEst": np.array([[0.5, 1.0], [1.5, 2.0]]),
                        "acceptedEqns": np.array([True, False, True]), "single": np.array([4.0])}])


def to_json(v):
    if isinstance(v, np.ndarray):
        return {"__array__": v.tolist(), "dtype": str(v.dtype)}
    if isinstance(v, np.generic):
        return v.item()
    if isinstance(v, dict):
        return {k: to_json(x) for k, x in v.items()}
    if isinstance(v, (list, tuple)):
        return [to_json(x) for x in v]
    return v


def main():
    from oracle.ref_harness import load_reference, _stubs_installed
    zr = load_reference(fp64=False)
    cwd = os.getcwd()
    os.chdir(HERE)
    try:
        with _stubs_installed():
            reg = zr.ImageRegistrator()
            for k, v in config_state().items():
                setattr(reg, k, v)
            reg.saveConfig("config_ref.zor")
            fresh = zr.ImageRegistrator()
            fresh.loadConfig("config_ref.zor")
    finally:
        os.chdir(cwd)
    loaded = {k: to_json(getattr(fresh, k, "<unset>")) for k in LOADED_ATTRS}
    with open(os.path.join(HERE, "config_ref_loaded.json"), "w") as fh:
        json.dump(loaded, fh, indent=1, sort_keys=True)
    print("wrote config_ref.zor and config_ref_loaded.json")


if __name__ == "__main__":
    main()

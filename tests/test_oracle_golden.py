"""The oracle restatement against golden fixtures made by the unmodified
reference (``tests/golden/make_golden.py``).  CPU only."""
import os

import numpy as np
import pytest

from oracle import zorro_oracle as zo
from tests.golden.make_golden import CASES, input_checksum
from zorro_gb300.synthetic import make_movie

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    path = os.path.join(GOLDEN, name + ".npz")
    return dict(np.load(path, allow_pickle=False))


def _subset(g, name, arr):
    arr = np.asarray(arr, dtype=np.float64).reshape(-1)
    return arr[g[name + "_idx"]], g[name + "_val"], float(np.sum(arr)), float(g[name + "_total"])


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    name = request.param
    g = _load(name)
    mv = make_movie(**CASES[name]["movie"])
    if input_checksum(mv["images"]) != str(g["checksum"]):
        pytest.skip("synthetic input differs on this platform; golden fixture not comparable")
    cap = {}
    res = zo.align_image_stack(mv["images"], capture=cap, **CASES[name]["attrs"])
    return name, g, res, cap


def test_tri_matrices(case):
    name, g, res, _ = case
    ed = res["errorDict"]
    for k in ("shiftsTriMat", "corrTriMat", "peaksigTriMat", "originTriMat"):
        np.testing.assert_allclose(np.asarray(ed[k], np.float64), g[k], rtol=1e-9, atol=1e-15, err_msg=k)


def test_translations_and_solver(case):
    name, g, res, _ = case
    np.testing.assert_allclose(res["translations"], g["translations"], rtol=0, atol=1e-9)
    ed = res["errorDict"]
    for k in ("weights", "errorX", "errorY", "relativeEst"):
        if k in g:
            np.testing.assert_allclose(np.asarray(ed[k]), g[k], rtol=1e-7, atol=1e-9, err_msg=k)
    for k in ("peaksigThres", "logisticK", "logisticNu"):
        if k in g:
            assert float(ed[k]) == pytest.approx(float(g[k]), rel=1e-9), k


def test_correlation_windows(case):
    name, g, res, cap = case
    for i, p in enumerate(g["cap_pairs"]):
        c = cap[tuple(int(v) for v in p)]
        for got, want in ((c["C"], g["cap_C_%d" % i]), (c["C_filt"], g["cap_Cfilt_%d" % i])):
            np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-12 * np.abs(want).max())


def test_sums_frc_dose(case):
    name, g, res, _ = case
    a, b, ta, tb = _subset(g, "imageSum", res["imageSum"])
    np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-6)
    assert ta == pytest.approx(tb, rel=1e-9)
    if "FRC" in g:
        np.testing.assert_allclose(res["FRC"], g["FRC"], rtol=1e-9, atol=1e-12, equal_nan=True)
    if "filtSum_idx" in g:
        a, b, ta, tb = _subset(g, "filtSum", res["filtSum"])
        np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-6)


def test_half_set_translations(case):
    name, g, res, _ = case
    if "transEven" not in g:
        pytest.skip("no independent half-set FRC in this case")
    np.testing.assert_allclose(res["transEven"], g["transEven"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(res["transOdd"], g["transOdd"], rtol=0, atol=1e-9)


def test_hot_pixel_counts(case):
    name, g, res, _ = case
    if "hot_guessHotpix" not in g:
        pytest.skip("no hot-pixel filter in this case")
    info = res["hotpixInfo"]
    for k in ("guessDeadpix", "guessHotpix", "neighborPix"):
        assert info[k] == int(g["hot_" + k]), k
    for k in ("cutoffLower", "cutoffUpper", "frameMean", "frameStd"):
        assert float(info[k]) == pytest.approx(float(g["hot_" + k]), rel=1e-12), k

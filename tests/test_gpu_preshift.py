"""preShift on the GPU (zorro.py:1089-1092, 1148-1168): the whole-plane peak
kernels (zr_full_*) against scipy / NumPy, and registrations against the
float64 oracle and the reference's own outputs (tests/golden/preshift.npz)."""
import ctypes as C
import os

import numpy as np
import pytest
import scipy.ndimage

from oracle import zorro_oracle as zo
from zorro_gb300 import _lib
from zorro_gb300 import hostmath as hm
from zorro_gb300.engine import _PEAK_DTYPE
from zorro_gb300.synthetic import make_movie

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _gpu(images, **attrs):
    from zorro_gb300.registrator import ImageRegistrator
    reg = ImageRegistrator()
    reg.images = images
    for k, v in attrs.items():
        setattr(reg, k, v)
    reg.alignImageStack()
    return reg


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_full_plane_kernels_match_scipy():
    import torch
    rng = np.random.default_rng(4)
    n, Cw, mS = 3, 64, 9
    planes = rng.normal(size=(n, Cw, Cw)).astype(np.float32)
    planes[1, 20, 41] += 9.0  # a clear peak inside the rolled disc
    dp = torch.from_numpy(planes.copy()).cuda()
    origin = torch.zeros(n, dtype=torch.float32, device="cuda")
    mean = torch.zeros(n, dtype=torch.float32, device="cuda")
    _lib.call("zr_full_prepare", dp.data_ptr(), n, Cw, 1, origin.data_ptr(), mean.data_ptr(), _stream())
    host = planes.copy()
    o = Cw // 2
    for p in range(n):
        assert origin[p].item() == host[p, o, o]
        c = host[p]
        c[o, o] = np.float32(0.125) * (c[o + 1, o] + c[o, o + 1] + c[o - 1, o] + c[o - 1, o] + c[o + 1, o + 1]
                                       + c[o - 1, o + 1] + c[o - 1, o + 1] + c[o - 1, o - 1])
    assert np.allclose(dp.cpu().numpy(), host, atol=1e-6)
    assert np.allclose(mean.cpu().numpy(), host.reshape(n, -1).mean(axis=1), atol=1e-6)
    sig = [0.0, 1.37, 3.0]
    taps = np.zeros((n, 2, 129), np.float32)
    rad = np.zeros((n, 2), np.int32)
    for p, s in enumerate(sig):
        t, r = hm.gaussian_taps(s)
        taps[p, :, :t.size] = t
        rad[p] = r
    dtaps, drad = torch.from_numpy(taps).cuda(), torch.from_numpy(rad).cuda()
    sel = torch.arange(n, dtype=torch.int32, device="cuda")
    filt = torch.zeros_like(dp)
    stats = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    wb = _lib.load().zr_full_work_bytes(n, Cw)
    work = torch.empty(wb, dtype=torch.uint8, device="cuda")
    _lib.call("zr_full_filter", dp.data_ptr(), n, Cw, sel.data_ptr(), n, dtaps.data_ptr(), drad.data_ptr(),
              mean.data_ptr(), filt.data_ptr(), stats.data_ptr(), work.data_ptr(), wb, _stream())
    F = filt.cpu().numpy()
    st = stats.cpu().numpy()
    m = mean.cpu().numpy()
    for p, s in enumerate(sig):
        ref = scipy.ndimage.gaussian_filter(host[p].astype(np.float64), s) if s > 0 else host[p].astype(np.float64)
        assert np.abs(F[p] - ref).max() < 2e-5, p
        d = F[p].astype(np.float64) - m[p]
        assert abs(st[p, 0] - d.sum()) < 1e-3 and abs(st[p, 1] - (d * d).sum()) < 1e-2 * max(1.0, (d * d).sum() * 1e-5)
        assert st[p, 2] == F[p].max()
    # masked argmax with rolled discs, peak significance, integer positions
    rolls = np.array([[0, 0], [-12, 9], [30, -31]], np.int32)
    drolls = torch.from_numpy(rolls).cuda()
    dsig = torch.from_numpy(np.array(sig, np.float64)).cuda()
    dnf = torch.zeros(n, dtype=torch.int32, device="cuda")
    res = torch.zeros((n, C.sizeof(_lib.PeakResult)), dtype=torch.uint8, device="cuda")
    _lib.call("zr_full_peaks", dp.data_ptr(), filt.data_ptr(), n, Cw, sel.data_ptr(), n, mS, drolls.data_ptr(),
              mean.data_ptr(), origin.data_ptr(), dsig.data_ptr(), dnf.data_ptr(), 16, res.data_ptr(),
              work.data_ptr(), wb, _stream())
    rec = np.frombuffer(res.cpu().numpy().tobytes(), dtype=_PEAK_DTYPE)
    disc = zo.preshift_mask([Cw, Cw], mS)
    for p in range(n):
        mk = np.roll(np.roll(disc, rolls[p, 0], axis=0), rolls[p, 1], axis=1)
        masked = F[p] * mk
        cy, cx = np.unravel_index(np.argmax(masked), masked.shape)
        assert (rec["cy"][p], rec["cx"][p]) == (cy, cx), p
        want = (masked[cy, cx] - F[p][mk].astype(np.float64).mean()) / F[p][mk].astype(np.float64).std()
        assert abs(rec["peaksig"][p] - want) < 1e-3 * max(1.0, abs(want))
    assert (rec["cy"][1], rec["cx"][1]) == (20, 41)


CASE_ATTRS = dict(shapePadded=[128, 128], fouCrop=[128, 128], maxShift=8, pixelsize=0.1, preShift=True,
                  doLazyFRC=False)


@pytest.mark.parametrize("mode", ["tri", "refine", "auto"])
def test_preshift_registration_against_oracle(mode):
    mv = make_movie(n_frames=8, shape=(120, 128), seed=23, mean_dose=3.0, drift_sigma=2.5)
    attrs = dict(CASE_ATTRS, triMode=mode)
    if mode == "auto":
        attrs.update(autoMax=4, peaksigThres=3.0)
    reg = _gpu(mv["images"].copy(), **attrs)
    ref = zo.align_image_stack(mv["images"], **attrs)
    ed, red = reg.errorDictList[-1], ref["errorDict"]
    tri = red["corrTriMat"] != 0
    assert np.array_equal(ed["corrTriMat"] != 0, tri)
    d = np.abs(ed["shiftsTriMat"] - red["shiftsTriMat"]).max(axis=2)[tri]
    assert np.mean(d < 1e-9) >= 0.9, d
    np.testing.assert_allclose(ed["peaksigTriMat"][tri], red["peaksigTriMat"][tri], rtol=2e-3, atol=2e-3)
    t = reg.translations - reg.translations.mean(axis=0)
    if mode == "tri":
        # 28 pairs make an ill-posed logistic weight fit (4 histogram bins), so
        # one 1/16 px pair flip may move the L1 optimum: the solve is checked
        # on the GPU's own measurements instead
        sol = zo.shifts_solver(ed["shiftsTriMat"], ed["corrTriMat"], ed["peaksigTriMat"], shapeImage=[128, 128],
                               maxShift=8, weightMode="autologistic", peaksigThres=6.0, logisticK=5.0,
                               logisticNu=0.15)
        ts = sol["translations"] - sol["translations"].mean(axis=0)
        assert np.abs(t - ts).max() <= 0.01 + 1e-9
    elif mode == "refine":
        tr = ref["translations"] - ref["translations"].mean(axis=0)
        assert np.mean(np.abs(t - tr).max(axis=1) <= 0.01 + 1e-9) >= 0.85


def test_preshift_against_reference_fixture():
    from tests.golden.make_golden import CASES
    g = np.load(os.path.join(GOLDEN, "preshift.npz"))
    case = CASES["preshift"]
    mv = make_movie(**case["movie"])
    reg = _gpu(mv["images"].copy(), **case["attrs"])
    ed = reg.errorDictList[-1]
    tri = g["corrTriMat"] != 0
    d = np.abs(ed["shiftsTriMat"] - g["shiftsTriMat"]).max(axis=2)[tri]
    assert np.mean(d < 1e-9) >= 0.9, d
    # the rolled search reaches shifts beyond the unrolled disc
    assert np.abs(g["shiftsTriMat"]).max() > case["attrs"]["maxShift"]

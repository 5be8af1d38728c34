"""GPU kernels against the oracle, one stage at a time (through the C ABI)."""
import numpy as np
import pytest

from oracle import zorro_oracle as zo
from zorro_gb300.synthetic import make_movie

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small():
    mv = make_movie(5, (100, 90), seed=2, mean_dose=3.0, drift_sigma=1.0)
    return mv["images"]


def crop_layout(F, P, C_):
    """The kernels' spectrum layout from a full P0 x P1 spectrum."""
    C0, C1 = C_
    rows = [r if r < C0 // 2 else P[0] - C0 + r for r in range(C0)] + [C0 // 2]
    return F[np.array(rows)][:, :C1 // 2 + 1]


@pytest.mark.parametrize("P,C_", [((128, 128), (64, 64)), ((128, 256), (128, 128)), ((256, 256), (256, 256)),
                                  ((1536, 1536), (768, 384)), ((1536, 3072), (1536, 3072))])
def test_spectra_match_numpy_fft(small, P, C_):
    from tests import gpu_helpers as gh
    G, S, GM, means, _ = gh.spectra(small, P, C_)
    N, H, W = small.shape
    np.testing.assert_allclose(means, small.reshape(N, -1).astype(np.float64).mean(axis=1), rtol=1e-5)
    m = np.zeros(P)
    m[:H, :W] = 1
    gm_ref = crop_layout(np.fft.fft2(m), P, C_)
    np.testing.assert_allclose(GM[:, :C_[1] // 2 + 1], gm_ref, atol=1e-4 * np.abs(gm_ref).max())
    for n in range(N):
        u = np.zeros(P)
        u[:H, :W] = small[n].astype(np.float64) - means[n]
        g_ref = crop_layout(np.fft.fft2(u), P, C_)
        s_ref = crop_layout(np.fft.fft2(u * u), P, C_)
        np.testing.assert_allclose(G[n][:, :C_[1] // 2 + 1], g_ref, atol=2e-6 * np.abs(g_ref).max() * np.sqrt(P[0] * P[1]) / 16)
        np.testing.assert_allclose(S[n][:, :C_[1] // 2 + 1], s_ref, atol=2e-6 * np.abs(s_ref).max() * np.sqrt(P[0] * P[1]) / 16)


@pytest.mark.parametrize("P,C_,mS", [((128, 128), (64, 64), 12), ((256, 256), (128, 128), 20),
                                     ((1536, 1536), (768, 384), 20), ((3072, 3072), (1536, 1536), 24)])
def test_correlation_windows_match_oracle(small, P, C_, mS):
    """C windows of mnxc2 (float32, mean-subtracted) vs the float64 oracle."""
    from tests import gpu_helpers as gh
    N = small.shape[0]
    _, _, _, _, dev = gh.spectra(small, P, C_)
    pairs = [(I, J) for I in range(N) for J in range(I + 1, N)]
    _, cw, _ = gh.windows(dev, N, C_, mS, pairs)
    dt = zo.Dtypes(True)
    padded, mask = zo.pad_stack(small, P)
    sC = np.array(C_)
    GM, MP = zo.mask_spectrum(mask, sC, dt)
    nc2 = zo.norm_const2(sC)
    spec = [zo.frame_spectra(padded[n], mask, sC, dt) for n in range(N)]
    for k, (I, J) in enumerate(pairs):
        ref, _ = zo.mnxc2(spec[I][0], spec[I][1], spec[J][0], spec[J][1], GM, MP, nc2, mS, suppressOrigin=False, dt=dt)
        scale = np.abs(ref).max()
        err = np.abs(cw[k] - ref).max() / scale
        assert err < 2e-5, (I, J, err)


def test_spectra_fill_their_pitch():
    """Every element of a spectrum buffer is written, the pitch padding of
    each column (rows C0 + 1 .. C0 + 3) as zeros: zr_pack_half scales each
    spectrum by its largest element, so stale memory there must not count."""
    import ctypes as C
    from tests import gpu_helpers as gh
    from zorro_gb300 import _lib
    torch = gh.torch_mod()
    lib = _lib.load()
    _lib.call("zr_init", torch.cuda.current_device())
    P, C_ = (256, 256), (128, 128)
    mv = make_movie(3, (200, 180), seed=4, mean_dose=1.5, drift_sigma=1.0)
    raw = gh.dev_tensor(mv["images"].astype(np.float32))
    fr = gh.frames_of(raw)
    se = lib.zr_spectrum_elems(C_[0], C_[1])
    K4 = lib.zr_spectrum_pitch(C_[1])
    G = torch.full((3, se, 2), 1e30, dtype=torch.float32, device="cuda")
    S = torch.full((3, se, 2), 1e30, dtype=torch.float32, device="cuda")
    wb = lib.zr_spectra_work_bytes(200, 3, C_[1])
    work = torch.full((wb,), 255, dtype=torch.uint8, device="cuda")
    _lib.call("zr_spectra", C.byref(fr), None, None, 0, 3, 0, P[0], P[1], C_[0], C_[1], G.data_ptr(), S.data_ptr(),
              work.data_ptr(), wb, gh.stream())
    torch.cuda.synchronize()
    for t in (G, S):
        a = t.cpu().numpy().reshape(3, K4, C_[0] + 4, 2)
        assert np.isfinite(a).all() and np.abs(a).max() < 1e20
        assert np.all(a[:, :, C_[0] + 1:, :] == 0.0)
    # the half-precision scales then come from the spectra themselves
    G16 = torch.zeros((3, se), dtype=torch.int32, device="cuda")
    sc = torch.zeros(3, dtype=torch.float32, device="cuda")
    pw = torch.zeros(16, dtype=torch.uint8, device="cuda")
    _lib.call("zr_pack_half", G.data_ptr(), 3, se, G16.data_ptr(), sc.data_ptr(), pw.data_ptr(), 16, gh.stream())
    torch.cuda.synchronize()
    m = np.abs(G.cpu().numpy().reshape(3, -1)).max(axis=1)
    s = sc.cpu().numpy()
    assert np.all(m * s < 2.0 ** 15) and np.all(m * s >= 2.0 ** 14), (m, s)


def test_peaks_match_oracle_on_same_windows(small):
    """locatePeak on the GPU vs the oracle, fed the same (GPU) windows."""
    from tests import gpu_helpers as gh
    P, C_, mS = (256, 256), (128, 128), 20
    N = small.shape[0]
    _, _, _, _, dev = gh.spectra(small, P, C_)
    pairs = [(I, J) for I in range(N) for J in range(I + 1, N)]
    _, cw, cw_dev = gh.windows(dev, N, C_, mS, pairs)
    res = gh.peaks(cw_dev, mS)
    mmask = zo.max_shift_mask(mS)
    dt = zo.Dtypes(True)
    agree = 0
    for k in range(len(pairs)):
        C = cw[k].astype(np.float64).copy()
        origin = C[mS, mS]
        C0 = np.fft.ifftshift(C)  # back to FFT order for the suppressOrigin stencil
        C0[0, 0] = 0.125 * (C0[1, 0] + C0[0, 1] + C0[-1, 0] + C0[-1, 0] + C0[1, 1] + C0[-1, 1] + C0[-1, 1] + C0[-1, -1])
        C = np.fft.fftshift(C0)
        r = zo.locate_peak(C, mmask, 16, "opti", dt=dt)
        assert res["origin"][k] == pytest.approx(origin, rel=1e-6)
        assert abs(res["sigma"][k] - r["sigma"]) < 0.02, (k, res["sigma"][k], r["sigma"])
        assert res["peaksig"][k] == pytest.approx(r["peaksig"], rel=1e-3)
        same = np.allclose([res["sy"][k], res["sx"][k]], r["shift"], atol=1e-9)
        agree += same
        if not same:
            assert np.abs(np.array([res["sy"][k], res["sx"][k]]) - r["shift"]).max() <= 1.0 / 16 + 1e-9
    assert agree >= len(pairs) - 1


@pytest.mark.parametrize("shape,binned", [((1400, 1300), (700, 650)), ((1100, 1030), (540, 520))])
def test_fourier_binning_matches_oracle(shape, binned):
    """zr_bin_fourier (Bluestein transforms of any length) against the
    float64 oracle's binStack."""
    import ctypes as C
    from tests import gpu_helpers as gh
    from zorro_gb300 import _lib
    torch = gh.torch_mod()
    lib = _lib.load()
    _lib.call("zr_init", torch.cuda.current_device())
    mv = make_movie(3, shape, seed=5, mean_dose=1.0, drift_sigma=1.0)
    raw = gh.dev_tensor(mv["images"].astype(np.float32))
    fr = gh.frames_of(raw)
    wb = lib.zr_bin_work_bytes(shape[0], shape[1], binned[0], binned[1])
    work = torch.empty(wb, dtype=torch.uint8, device="cuda")
    out = torch.zeros((3, binned[0], binned[1]), dtype=torch.float32, device="cuda")
    _lib.call("zr_bin_fourier", C.byref(fr), binned[0], binned[1], out.data_ptr(), work.data_ptr(), wb, gh.stream())
    torch.cuda.synchronize()
    ref = zo.bin_stack(mv["images"].astype(np.float32), binned, zo.Dtypes(True))
    got = out.cpu().numpy()
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 2e-5, err


@pytest.mark.parametrize("shape,binned", [((8184, 11520), (4092, 5760)), ((11520, 8184), (5760, 4092))])
def test_fourier_binning_superres(shape, binned):
    """Four K3 super-resolution frames (11520 x 8184, either orientation)
    binned 2x to 5760 x 4092 against the float64 oracle's binStack: the
    11520-point side transformed directly by the mixed-radix engine (a
    Bluestein convolution would need 32768 points), the 8184-point side and
    the binned sides by Bluestein."""
    import ctypes as C
    import os
    from tests import gpu_helpers as gh
    from zorro_gb300 import _lib
    torch = gh.torch_mod()
    lib = _lib.load()
    _lib.call("zr_init", torch.cuda.current_device())
    mv = make_movie(4, shape, seed=41, mean_dose=0.25, drift_sigma=1.0)
    raw = gh.dev_tensor(mv["images"].astype(np.float32))
    fr = gh.frames_of(raw)
    wb = lib.zr_bin_work_bytes(shape[0], shape[1], binned[0], binned[1])
    work = torch.empty(wb, dtype=torch.uint8, device="cuda")
    out = torch.zeros((4, binned[0], binned[1]), dtype=torch.float32, device="cuda")
    _lib.call("zr_bin_fourier", C.byref(fr), binned[0], binned[1], out.data_ptr(), work.data_ptr(), wb, gh.stream())
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    del raw, work, out
    ref = zo.bin_stack(mv["images"], binned, zo.Dtypes(True, os.cpu_count() or 1))
    err = np.abs(got - ref).max() / np.abs(ref).max()
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    print("%s -> %s: max err %.2e of max, rel L2 %.2e" % (shape, binned, err, rel))
    assert err < 2e-5 and rel < 1e-5, (err, rel)


def test_fourier_binning_refuses_unsupported_long_sides():
    """A side above 8192 that the engine cannot transform directly (and whose
    Bluestein convolution does not fit one CTA) is refused with ZR_ESIZE."""
    import ctypes as C
    from tests import gpu_helpers as gh
    from zorro_gb300 import _lib
    torch = gh.torch_mod()
    lib = _lib.load()
    raw = torch.zeros((1, 600, 9000), dtype=torch.float32, device="cuda")
    fr = gh.frames_of(raw)
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    rc = lib.zr_bin_fourier(C.byref(fr), 520, 4500, C.c_void_p(dummy.data_ptr()), C.c_void_p(dummy.data_ptr()),
                            C.c_size_t(1 << 40), None)
    assert rc == -3
    assert "9216" in _lib.last_error()


def _stream():
    import ctypes
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_histogram_matches_numpy():
    """zr_histogram against np.histogram (hotpixFilter's histogram,
    zorro.py:2530-2533): unit bins from a half-integer edge (float32 path)
    and from another edge (float64 path), values on and next to every edge."""
    import torch
    from zorro_gb300 import _lib
    rng = np.random.default_rng(5)
    v = rng.poisson(20.0, 300000).astype(np.float32) * rng.uniform(0.9, 1.1, 300000).astype(np.float32)
    extra = []
    for h in np.arange(-3.5, 60.5, 0.5, dtype=np.float32):
        extra += [h, np.nextafter(h, np.float32(-np.inf)), np.nextafter(h, np.float32(np.inf))]
    extra += [-1e-30, -0.0, 0.0, np.inf, -np.inf, np.nan, 3e9, -0.50000006, -0.49999997]
    v = np.concatenate([v, np.array(extra, np.float32)])
    dv = torch.from_numpy(v).cuda()
    for e0, nb in [(-0.5, 45), (4.5, 40), (0.25, 50)]:
        edges = e0 + np.arange(nb + 1, dtype=np.float64)
        want, _ = np.histogram(v[np.isfinite(v)], edges)
        h = torch.zeros(nb, dtype=torch.int32, device="cuda")
        _lib.call("zr_histogram", dv.data_ptr(), v.size, e0, nb, h.data_ptr(), _stream())
        assert np.array_equal(h.cpu().numpy(), want), e0


def test_hotpix_maps_match_oracle():
    """zr_hotpix_maps on the oracle's unaligned sum with the oracle's fit:
    dead/hot/neighbourly counts exact; logisticMask and the fill map
    (singleton PSF fill + neighbourFilt) within float32 rounding.  The movie
    has a dead strip on the top rows and the right columns and a hot cluster,
    so that many pixels take the neighbour branch (also at the edges)."""
    import torch
    from zorro_gb300 import _lib
    from zorro_gb300._lib import HotpixParams
    mv = make_movie(12, (203, 190), seed=9, mean_dose=2.0, drift_sigma=0.5, dtype="uint8", gain_map=True,
                    hot_fraction=3e-3)
    imgs = mv["images"].copy()
    imgs[:, :3, :] = 0.0
    imgs[:, :, -2:] = 0.0
    imgs[:, 100:105, 40:46] *= 8.0
    info0 = dict(zo.DEFAULTS["hotpixInfo"])
    _, info, maps = zo.hotpix_filter(imgs.copy(), info0, dt=zo.Dtypes(True))
    usum = maps["unalignedSum"].astype(np.float32)
    fit = maps["fit"]
    m, H, W = imgs.shape
    prm = HotpixParams()
    prm.mu, prm.sigma = float(fit["mu"]), float(fit["sigma"])
    prm.cutoff_lower, prm.cutoff_upper = float(fit["cutoffLower"]), float(fit["cutoffUpper"])
    prm.logistic_k, prm.relax = float(np.float32(info0["logisticK"])), float(np.float32(info0["relax"]))
    psf = zo.psf_kernel("K2", zo.Dtypes(True)).ravel()
    for i in range(9):
        prm.psf[i] = float(psf[i])
    prm.neighbour_thres = 0.01
    prm.best_mean = float(fit["mu"] / m)
    lib = _lib.load()
    du = torch.from_numpy(usum).cuda()
    ha = torch.zeros((H, W), dtype=torch.float32, device="cuda")
    hb = torch.zeros((H, W), dtype=torch.float32, device="cuda")
    cnt = torch.zeros(4, dtype=torch.int32, device="cuda")
    wb = lib.zr_hotpix_work_bytes(H, W)
    work = torch.empty(wb, dtype=torch.uint8, device="cuda")
    import ctypes
    _lib.call("zr_hotpix_maps", du.data_ptr(), H, W, m, ctypes.byref(prm), ha.data_ptr(), hb.data_ptr(),
              cnt.data_ptr(), work.data_ptr(), wb, _stream())
    c = cnt.cpu().numpy()
    assert (int(c[0]), int(c[1]), int(c[2])) == (info["guessDeadpix"], info["guessHotpix"], info["neighborPix"])
    assert info["neighborPix"] > 500 and info["guessDeadpix"] > 500
    np.testing.assert_allclose(ha.cpu().numpy(), maps["logisticMask"], rtol=0, atol=2e-6)
    b_ref = maps["singleton"] * maps["psfFiltMean"] + maps["neighbourFilt"]
    np.testing.assert_allclose(hb.cpu().numpy(), b_ref, rtol=0, atol=2e-6 * max(1.0, float(np.abs(b_ref).max())))


@pytest.mark.parametrize("rtype,shape", [(0, (64, 60)), (1, (64, 60)), (2, (64, 60)), (3, (64, 60)),
                                         (1, (63, 61)), (2, (65, 59)), (3, (63, 61))])
@pytest.mark.parametrize("gdiv", [0.0, 3.0])
def test_gain_sum_every_raw_type(rtype, shape, gdiv):
    """zr_gain_sum against the frame-ordered float32 sum of
    float32(gain * raw) (/ gdiv): every raw type, the vector path (H*W % 4 ==
    0) and the per-pixel path; the float64 total within rounding."""
    import ctypes
    import torch
    from zorro_gb300 import _lib
    from zorro_gb300._lib import Frames
    rng = np.random.default_rng(rtype * 10 + shape[1])
    N, (H, W) = 11, shape
    np_t = {0: np.float32, 1: np.uint8, 2: np.uint16, 3: np.float16}[rtype]
    raw = rng.poisson(3.0, (N, H, W)).astype(np_t)
    if rtype in (0, 3):
        raw = (raw + rng.uniform(0, 1, (N, H, W))).astype(np_t)
    gain = rng.uniform(0.8, 1.2, (H, W)).astype(np.float32)
    want = np.zeros((H, W), np.float32)
    for n in range(N):
        v = gain * raw[n].astype(np.float32)
        if gdiv:
            v = v / np.float32(gdiv)
        want = want + v
    draw = torch.from_numpy(raw.view(np.int16) if rtype == 2 else raw).cuda()  # the same bytes
    dgain = torch.from_numpy(gain).cuda()
    fr = Frames()
    fr.raw, fr.raw_type, fr.gain, fr.hot_a, fr.hot_b = draw.data_ptr(), rtype, dgain.data_ptr(), None, None
    fr.gain_divisor, fr.n_frames, fr.height, fr.width, fr.frame_stride = gdiv, N, H, W, H * W
    out = torch.zeros((H, W), dtype=torch.float32, device="cuda")
    tot = torch.zeros(1, dtype=torch.float64, device="cuda")
    _lib.call("zr_gain_sum", ctypes.byref(fr), out.data_ptr(), tot.data_ptr(), _stream())
    assert np.array_equal(out.cpu().numpy(), want)
    assert abs(tot.item() - want.astype(np.float64).sum()) <= 1e-9 * abs(want.astype(np.float64).sum())

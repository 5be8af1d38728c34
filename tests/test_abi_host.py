"""CPU-only checks: the C ABI library loads and exports every symbol the
header declares, and the host-side float64 steps of the product agree with
the oracle.  No kernel is launched here."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import zorro_oracle as zo
from zorro_gb300 import hostmath as hm

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "zorro_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(zr_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from zorro_gb300 import _lib
    from zorro_gb300.build import build
    build()
    return _lib.load()


def test_library_exports_every_header_symbol(lib):
    from zorro_gb300 import _lib
    names = header_functions()
    assert names, "no declarations parsed"
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_lib.EXPORTS), set(names) ^ set(_lib.EXPORTS)


def test_size_queries(lib):
    assert lib.zr_version() >= 100
    assert lib.zr_spectrum_pitch(2048) == 1028
    assert lib.zr_spectrum_elems(2048, 2048) == 2052 * 1028
    assert lib.zr_xcorr_work_bytes(10, 2048, 100) == 10 * 201 * 1028 * 8


def test_errors_are_reported_without_a_gpu(lib):
    from zorro_gb300 import _lib
    rc = lib.zr_locate_peaks(None, 1, 100, None, None, None)
    assert rc == -1
    assert "null" in _lib.last_error()


def _ordered_neighbours(v, k):
    """The k float32 values on each side of v (and v) in float32 order."""
    u = np.array([v], np.float32).view(np.uint32)[0]
    key = int(~u & 0xffffffff) if u & 0x80000000 else int(u | 0x80000000)
    keys = np.arange(key - k, key + k + 1, dtype=np.int64)
    keys = keys[(keys >= 0) & (keys <= 0xffffffff)].astype(np.uint32)
    bits = np.where(keys & 0x80000000, keys & 0x7fffffff, ~keys).astype(np.uint32)
    return bits.view(np.float32)


def test_hotpix_thresholds_give_the_counts_of_the_quotient(lib):
    """zr_hotpix_thresholds (host code of zr_hotpix_maps): counting float32
    sums against the two float32 thresholds gives exactly the dead/hot
    decisions of the float64 quotient (s - mu) / sigma < cutoffLower and
    > cutoffUpper (zorro.py:2595-2601), on and around the thresholds, over a
    sweep of values and at +-0, +-inf and NaN; sigma 0 included."""
    import ctypes
    from zorro_gb300 import _lib
    rng = np.random.default_rng(6)
    cases = [(31.396991311237343, 5.654671154694482, -4.0, 2.4724910259246826), (24.5, 0.0, -1.9, -0.25),
             (1.0286607132473808, 1.2334786214509157, -4.0, 0.9497635), (2.5e5, 480.0, -3.3, 3.25)]
    cases += [(float(rng.uniform(0, 100)), float(rng.uniform(0.3, 9)), float(np.float32(rng.uniform(-5, -1))),
               float(np.float32(rng.uniform(-1, 4)))) for _ in range(20)]
    for mu, sigma, cl, cu in cases:
        sd, sh = ctypes.c_float(), ctypes.c_float()
        _lib.call("zr_hotpix_thresholds", mu, sigma, cl, cu, ctypes.byref(sd), ctypes.byref(sh))
        s_dead, s_hot = np.float32(sd.value), np.float32(sh.value)
        vals = [_ordered_neighbours(s_dead, 3000), np.array([mu], np.float32),
                (mu + sigma * rng.normal(0, 4, 200000)).astype(np.float32),
                np.array([0.0, -0.0, np.inf, -np.inf, np.nan], np.float32)]
        if np.isfinite(s_hot):
            vals.append(_ordered_neighbours(s_hot, 3000))
        s = np.concatenate(vals)
        with np.errstate(all="ignore"):
            q = (s.astype(np.float64) - mu) / sigma
            assert np.array_equal(s < s_dead, q < np.float64(np.float32(cl))), (mu, sigma, cl)
            assert np.array_equal(s >= s_hot, q > np.float64(np.float32(cu))), (mu, sigma, cu)
    with pytest.raises(ValueError):
        _lib.call("zr_hotpix_thresholds", 1.0, -1.0, -4.0, 3.0, ctypes.byref(ctypes.c_float()),
                  ctypes.byref(ctypes.c_float()))


@pytest.mark.parametrize("mode,w", [("tri", 5), ("diag", 3), ("diag", 1), ("first", 5), ("auto", 5)])
def test_tri_indices_and_equation_matrix(mode, w):
    for N in (2, 7, 40):
        t = hm.tri_indices(N, mode, w, 0)
        assert np.array_equal(t, zo.tri_indices(N, mode, w, 0))
        if mode != "first" and N > 1:
            r = t[:-1, 1:]
            assert np.array_equal(hm.equation_matrix(r), zo.solver_matrix(r))


def test_shift_kernels_match_reference_kernel():
    rng = np.random.default_rng(0)
    t = rng.normal(0, 3, size=(20, 2))
    for (ry, rx, ap, ky, kx), tt in zip(hm.shift_params(t), t):
        assert (ry, rx) == tuple(np.round(tt).astype(int))
        k2 = zo.lanczos_kernel(np.remainder(tt, 1))
        if ap:
            np.testing.assert_allclose(np.outer(ky, kx), k2, rtol=1e-12, atol=1e-15)


def test_shift_table_matches_per_frame_records():
    """shift_table (all frames at once) gives the bytes of the zr_shift_t
    records built frame by frame from shift_params, for float64, float32 and
    integer translations, and for the integer-roll-only case."""
    import ctypes
    from zorro_gb300._lib import Shift
    assert hm.SHIFT_DTYPE.itemsize == ctypes.sizeof(Shift)
    rng = np.random.default_rng(2)
    H, W = 3838, 3710
    for trial in range(60):
        n = int(rng.integers(1, 50))
        t = rng.normal(0, 5, (n, 2))
        if trial % 3 == 0:
            t = np.round(t * 16) / 16
        if trial % 4 == 0:
            t[::3] = np.round(t[::3])
        if trial % 5 == 0:
            t = t.astype(np.float32)
        if trial % 7 == 0:
            t = np.round(t).astype(int)
        sh = (Shift * n)()
        for k, (ry, rx, ap, ky, kx) in enumerate(hm.shift_params(t)):
            sh[k].roll_y, sh[k].roll_x, sh[k].apply = ry % H, rx % W, ap
            for i in range(3):
                sh[k].ky[i] = float(ky[i])
                sh[k].kx[i] = float(kx[i])
        assert bytes(sh) == hm.shift_table(t, H, W).tobytes(), trial
        rolls = hm.shift_table(t, H, W, lanczos=False)
        assert np.array_equal(rolls["roll_y"], np.round(t[:, 0]).astype(int) % H)
        assert np.array_equal(rolls["roll_x"], np.round(t[:, 1]).astype(int) % W)
        assert not rolls["apply"].any() and (rolls["ky"] == [0, 1, 0]).all() and (rolls["kx"] == [0, 1, 0]).all()


def test_frc_tiles_match_oracle():
    rng = np.random.default_rng(1)
    for shape in ((800, 800), (3838, 3710), (1024, 1024)):
        t = rng.normal(0, 4, size=(10, 2))
        t -= t.mean(axis=0)
        offs, tiles = hm.frc_tiles(shape, t)
        crop = zo.frc_crop_limits(t)
        assert tiles[0] * tiles[1] == len(offs)
        if len(offs):
            assert offs[0, 0] == int(crop[0]) and offs[0, 1] == int(crop[1])


def test_dose_constants_match_oracle():
    dt = zo.Dtypes(True)
    for P, ps, dose in (((1024, 1024), 0.1, 1.0), ((4096, 4096), 0.105, 1.2 * 1.05 ** 2)):
        p = [dose, 0.24499, -1.6649, 2.8141, 32, 0]
        a = hm.dose_constants(40, P, ps, 300.0, p)
        b = zo.dose_filter_params(40, P, ps, 300.0, p, dt=dt)
        np.testing.assert_allclose(a["thresQ"], b["thresQ"], rtol=1e-12)
        np.testing.assert_allclose(a["dose_end"], b["accum"][1:], rtol=1e-12)


def test_hotpix_fit_matches_oracle():
    from zorro_gb300.synthetic import make_movie
    mv = make_movie(20, (128, 120), seed=11, mean_dose=1.6, dtype="uint8", gain_map=True, hot_fraction=1e-3)
    usum = np.sum(mv["images"], axis=0)
    info = dict(zo.DEFAULTS["hotpixInfo"])
    ref = zo.hotpix_fit(usum, info, 20, zo.Dtypes(True))
    sm, ps, edges = hm.hotpix_bins(np.float64(np.sum(usum, dtype=np.float64)) / usum.size, info["maxSigma"])
    hist, _ = np.histogram(usum, edges)
    mu, sg, cl, cu, _ = hm.hotpix_fit(hist, edges, sm, ps, info)
    assert mu == pytest.approx(ref["mu"], rel=1e-6)
    assert sg == pytest.approx(ref["sigma"], rel=1e-6)
    assert cl == ref["cutoffLower"] or (np.isnan(cl) and np.isnan(ref["cutoffLower"]))
    assert cu == pytest.approx(float(ref["cutoffUpper"]), rel=1e-5)


def test_numpy_axis0_sum_is_sequential():
    """The hot-pixel kernel sums frames in order in float32, which is what
    np.sum(stack, axis=0) does for a float32 stack."""
    rng = np.random.default_rng(3)
    a = (rng.random((40, 64, 64)) * 3).astype(np.float32)
    s = np.zeros((64, 64), np.float32)
    for k in range(40):
        s = s + a[k]
    assert np.array_equal(np.sum(a, axis=0), s)


def _numpy_exp_pow_are_libm():
    import math
    rng = np.random.default_rng(2)
    x = rng.uniform(-700, 700, 20000)
    v, e = rng.uniform(1, 1e6, 20000), rng.uniform(0.05, 5, 20000)
    return (np.array_equal(np.exp(x), [math.exp(t) for t in x]) and
            np.array_equal(v ** e, [math.pow(a, b) for a, b in zip(v, e)]))


def test_logistic_fit_matches_scipy_nelder_mead():
    """zr_logistic_fit returns scipy's Nelder-Mead point bit for bit on the
    logistic-CDF objective (ties and small bin counts included) where NumPy's
    exp and pow are the C library's (aarch64); NumPy's SIMD exp/pow on x86
    differ in the last bit for a few percent of arguments, which moves the
    simplex path."""
    import scipy.optimize
    if not _numpy_exp_pow_are_libm():
        pytest.skip("NumPy's exp/pow are not the C library's on this platform")
    rng = np.random.default_rng(5)
    for trial in range(60):
        n = int(rng.choice([15, 28, 45, 190, 780]))
        ps = np.abs(rng.normal(rng.uniform(5, 40), rng.uniform(1, 10), n)) + 0.01
        if trial % 5 == 0:
            ps = np.round(ps)
        pdf, edges = np.histogram(ps, bins=int(ps.size / 7.0))
        h = edges[:-1]
        cdf = np.cumsum(pdf.astype("float32"))
        cdf /= cdf[-1]
        with np.errstate(over="ignore"):
            r = scipy.optimize.minimize(zo._logistic_cdf_error64, (np.mean(ps), 5.0, 1.0), args=(h, cdf),
                                        method="Nelder-Mead", bounds=((np.min(ps), np.max(ps)), (0.1, 20.0), (0.05, 5.0)),
                                        options={"xatol": 1e-10, "fatol": 1e-14, "maxiter": 4000, "maxfev": 8000})
        x = hm.logistic_nelder_mead(h, cdf, (np.mean(ps), 5.0, 1.0), (np.min(ps), 0.1, 0.05), (np.max(ps), 20.0, 5.0))
        assert np.array_equal(x, r.x), (trial, x, r.x)


def test_logistic_fit_converges_to_a_minimum():
    """On every platform: the native fit ends on a point whose objective is
    no worse than scipy's by more than the stopping tolerance on well-posed
    problems (hundreds of peaks)."""
    import scipy.optimize
    rng = np.random.default_rng(9)
    for trial in range(10):
        ps = np.abs(rng.normal(rng.uniform(10, 40), rng.uniform(2, 8), 780)) + 0.01
        pdf, edges = np.histogram(ps, bins=int(ps.size / 7.0))
        h = edges[:-1]
        cdf = np.cumsum(pdf.astype("float32"))
        cdf /= cdf[-1]
        x = hm.logistic_nelder_mead(h, cdf, (np.mean(ps), 5.0, 1.0), (np.min(ps), 0.1, 0.05), (np.max(ps), 20.0, 5.0))
        with np.errstate(over="ignore"):
            r = scipy.optimize.minimize(zo._logistic_cdf_error64, (np.mean(ps), 5.0, 1.0), args=(h, cdf),
                                        method="Nelder-Mead", bounds=((np.min(ps), np.max(ps)), (0.1, 20.0), (0.05, 5.0)),
                                        options={"xatol": 1e-10, "fatol": 1e-14, "maxiter": 4000, "maxfev": 8000})
            fx = zo._logistic_cdf_error64(x, h, cdf)
        assert fx <= r.fun * (1 + 1e-6) + 1e-9, (trial, fx, r.fun)


def test_hotpix_fit_bit_exact_over_random_histograms():
    """The product's CDF fit (L-BFGS-B with the forward-difference gradient
    passed in) returns the oracle's scipy L-BFGS-B result bit for bit."""
    rng = np.random.default_rng(3)
    info = dict(zo.DEFAULTS["hotpixInfo"])
    for t in range(12):
        usum = rng.poisson(rng.uniform(5, 60), (200, 150)).astype(np.float32)
        if t % 3 == 0:
            usum[rng.random(usum.shape) < 1e-3] *= 20
        if t % 4 == 0:
            usum[rng.random(usum.shape) < 1e-3] = 0
        mean = float(np.sum(usum, dtype=np.float64)) / usum.size
        sm, ps, edges = hm.hotpix_bins(mean, info["maxSigma"])
        hist, _ = np.histogram(usum, edges)
        mu, sg, cl, cu, _ = hm.hotpix_fit(hist, edges, sm, ps, dict(info))
        ref = zo.hotpix_fit(usum, dict(info), 20, zo.Dtypes(True))
        assert mu == ref["mu"] and sg == ref["sigma"], t
        assert cu == ref["cutoffUpper"], t
        assert cl == ref["cutoffLower"] or (np.isnan(cl) and np.isnan(ref["cutoffLower"])), t


@pytest.mark.parametrize("info", [{"Horizontal": True, "Vertical": True, "Diagonal": False},
                                  {"Horizontal": True, "Vertical": False, "Diagonal": False},
                                  {"Horizontal": False, "Vertical": True, "Diagonal": True},
                                  {"Horizontal": False, "Vertical": False, "Diagonal": True}])
def test_gain_reference_orientation(info):
    """loadGainRef orients the gain reference as loadData does
    (zorro.py:3486-3502)."""
    from zorro_gb300.registrator import ImageRegistrator
    g = np.arange(12, dtype=np.float32).reshape(3, 4)
    want = np.rot90(g, 1) if info["Diagonal"] else g
    if info["Horizontal"] and info["Vertical"]:
        want = np.rot90(want, 2)
    elif info["Horizontal"]:
        want = want[:, ::-1]
    elif info["Vertical"]:
        want = want[::-1, :]
    r = ImageRegistrator()
    r.gainInfo = dict(info)
    assert np.array_equal(r.loadGainRef(g), want)


def test_struct_layouts_match_the_header(tmp_path):
    """Every struct of include/zorro_gb300.h has the size and field offsets
    of its ctypes mirror (a C program built against the header prints them)."""
    import shutil
    import subprocess
    from zorro_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = {"zr_frames_t": _lib.Frames, "zr_hotpix_params_t": _lib.HotpixParams, "zr_peak_params_t": _lib.PeakParams,
             "zr_peak_result_t": _lib.PeakResult, "zr_shift_t": _lib.Shift, "zr_dose_params_t": _lib.DoseParams,
             "zr_plan_shape_t": _lib.PlanShape, "zr_plan_choice_t": _lib.PlanChoice,
             "zr_batch_limits_t": _lib.BatchLimits, "zr_batch_movie_t": _lib.BatchMovie}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "zorro_gb300.h"', "int main(void) {"]
    for cname, cls in pairs.items():
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in cls._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-I", inc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for ln in out:
        p = ln.split()
        if len(p) == 3:
            got[(p[0], p[1])] = int(p[2])
    for cname, cls in pairs.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)

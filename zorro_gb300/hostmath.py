"""Host-side float64 steps of the registration path.

These are the small, sequential pieces of ``alignImageStack`` that the
reference also runs on the host with NumPy/SciPy: the pair triangle, the
weighted-L1 drift solve and its logistic weights, the per-frame shift
kernels, the FRC tile grid, the dose-filter constants and the normal-CDF fit
of the hot-pixel histogram.  Each function names the reference lines it
follows.  The GPU does every pass over pixels.
"""
from __future__ import annotations

import concurrent.futures
import functools
import math
import threading

import numpy as np
import scipy.optimize
import scipy.special
import scipy.stats

# The reference's logistic fit and drift solve call the stochastic
# scipy.optimize.basinhopping without a seed (zorro.py:1415,1422,2008).  Here
# the drift solve is the exact weighted-L1 optimum of the same objective and
# the logistic fit a deterministic Nelder-Mead search, so results repeat.


def tri_indices(N, triMode="diag", diagWidth=5, diagStart=0):
    """Pairs to correlate, [N,N] bool ([1,N] for 'first').  zorro.py:558-579."""
    x = np.arange(N)
    trimesh = x[None, :] - x[:, None]
    if triMode == "first":
        t = np.ones([1, N], dtype=bool)
        t[0, 0] = False
        return t
    if triMode == "diag":
        if diagWidth is None or diagWidth < 0:
            diagWidth = N
        return (trimesh <= diagWidth + diagStart) & (trimesh > diagStart)
    if triMode in ("autocorr", "refine"):
        return trimesh == 0
    return trimesh >= 1


def pair_list(tri):
    """(I, J) in the reference's loop order (rows, then columns)."""
    I, J = np.nonzero(tri)
    return np.stack([I, J], axis=1).astype(np.int32)


def equation_matrix(tri):
    """Relative-drift equation matrix, one row per pair.  zorro.py:1292-1311:
    row I contributes the 180-degree rotation of tri[I:last, I:last]."""
    N = tri.shape[0]
    last = np.zeros(N, dtype=int)
    M = 0
    for I in range(N):
        nz = np.nonzero(tri[I])[0]
        if nz.size:
            last[I] = nz[-1] + 1
            M += last[I] - I
    A = np.zeros([int(M), N])
    pos = 0
    for I in range(N):
        blk = tri[I:last[I], I:last[I]][::-1, ::-1]
        A[pos:pos + blk.shape[0], I:I + blk.shape[1]] = blk
        pos += blk.shape[0]
    return A


def l1_solve(A, b, w, lo, hi):
    """argmin_x sum(w * |A x - b|) with lo <= x <= hi (the objective of
    zorro_util.py:849-851), exactly.  The native simplex of libzorrogb
    (zr_l1_solve) solves the dual linear programme (max b.y s.t. A^T y = 0,
    |y| <= w), whose equality multipliers are the primal optimum.  If that
    point leaves the box, the bounded primal LP is solved instead."""
    import ctypes as C
    from . import _lib
    m, n = A.shape
    w = np.ascontiguousarray(w, dtype=np.float64)
    Ac = np.ascontiguousarray(A, dtype=np.float64)
    bc = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(n)
    st = C.c_int(-1)
    rc = _lib.load().zr_l1_solve(Ac.ctypes.data, bc.ctypes.data, w.ctypes.data, m, n, float(lo), float(hi),
                                 x.ctypes.data, C.byref(st))
    if rc == 0 and st.value == 0:
        return x
    cost = np.concatenate([np.zeros(n), w])
    eye = np.eye(m)
    A_ub = np.block([[A, -eye], [-A, -eye]])
    b_ub = np.concatenate([b, -b])
    bounds = [(lo, hi)] * n + [(0.0, None)] * m
    res = scipy.optimize.linprog(cost, A_ub=A_ub, b_ub=b_ub, bounds=bounds, method="highs")
    if not res.success:
        raise RuntimeError("drift solve failed: %s" % res.message)
    return res.x[:n]


def logistic_nelder_mead(hSigma, cdf, x0, lo, hi, xatol=1e-10, fatol=1e-14, maxiter=4000, maxfev=8000):
    """Bounded Nelder-Mead on the logistic-CDF error (zr_logistic_fit, host
    C++): the steps of scipy.optimize.minimize(method='Nelder-Mead',
    bounds=...), so it returns scipy's point wherever NumPy's exp and pow are
    the C library's (as on aarch64)."""
    import ctypes as C
    from . import _lib
    h = np.ascontiguousarray(hSigma, dtype=np.float64)
    c = np.ascontiguousarray(cdf, dtype=np.float32)
    a0, alo, ahi = (np.ascontiguousarray(v, dtype=np.float64) for v in (x0, lo, hi))
    x = np.zeros(3)
    _lib.call("zr_logistic_fit", h.ctypes.data, c.ctypes.data, len(h), a0.ctypes.data, alo.ctypes.data,
              ahi.ctypes.data, float(xatol), float(fatol), int(maxiter), int(maxfev), x.ctypes.data, None, None)
    return x


def logistic_fit(peaksigTriMat):
    """Logistic fit to the CDF of peak significances.  zorro.py:1981-2022.

    The reference minimises the error with unseeded basinhopping, which
    returns a different point on every run.  Here the same objective is
    minimised from the reference's start point (mean, 5, 1) within the same
    bounds by Nelder-Mead to tight tolerances, so the fit repeats and moves
    continuously with its input."""
    ps = peaksigTriMat[peaksigTriMat > 0.0]
    bins = int(ps.size / 7.0)
    if bins <= 0:
        raise ValueError("autologistic weights need at least 7 positive peak significances (got %d)" % ps.size)
    pdf, edges = np.histogram(ps, bins=bins)
    hSigma = edges[:-1]
    pdf = pdf.astype("float32")
    cdf = np.cumsum(pdf)
    cdf /= cdf[-1]
    x = logistic_nelder_mead(hSigma, cdf, (np.mean(ps), 5.0, 1.0), (np.min(ps), 0.1, 0.05), (np.max(ps), 20.0, 5.0))
    return {"peaksigThres": x[0], "logisticK": x[1], "logisticNu": x[2], "pdfPeaks": pdf, "cdfPeaks": cdf,
            "hSigma": hSigma}


_L1_POOL = None
_L1_LOCK = threading.Lock()


def _l1_pool():
    """Threads for the y-axis solves (the native solver releases the GIL),
    kept for the process."""
    global _L1_POOL
    with _L1_LOCK:
        if _L1_POOL is None:
            _L1_POOL = concurrent.futures.ThreadPoolExecutor(4, thread_name_prefix="zorro-l1")
        return _L1_POOL


def solve_shifts(shiftsTriMat_in, corrTriMat_in, peaksigTriMat_in, *, shapeImage, maxShift, weightMode,
                 peaksigThres, logisticK, logisticNu, defer_errors=False):
    """The drift solve and its error analysis.  zorro.py:1260-1567.
    Returns the errorDict (its 'translations' are the frame shifts to apply).
    With ``defer_errors`` it returns (errorDict so far, translations,
    finish): the caller can use the translations at once and call finish()
    later to add the error analysis (the same values, in the same order)."""
    sh = shiftsTriMat_in[:-1, 1:, :]
    co = corrTriMat_in[:-1, 1:]
    ps = peaksigTriMat_in[:-1, 1:]
    tri = co.astype(bool)
    ed = {"corrTriMat": corrTriMat_in, "peaksigTriMat": peaksigTriMat_in}
    N = shiftsTriMat_in.shape[0] - 1
    A = equation_matrix(tri)
    M = A.shape[0]
    where = np.nonzero(tri.ravel())[0]
    unrav = np.unravel_index(where, [N, N])
    b_x = sh[tri, 1].ravel()
    b_y = sh[tri, 0].ravel()
    accepted = np.ones_like(b_x, dtype=bool)
    pk = ps[tri].ravel()
    if weightMode is None or weightMode == "corr":
        weights = pk
    elif weightMode == "unweighted":
        weights = np.ones_like(pk)
    elif weightMode in ("norm", "normalized"):
        weights = (pk - pk.min()) / (pk.max() - pk.min())
    elif weightMode in ("autologistic", "logistic"):
        if weightMode == "autologistic":
            fit = logistic_fit(peaksigTriMat_in)
            ed.update(fit)
            peaksigThres, logisticK, logisticNu = fit["peaksigThres"], fit["logisticK"], fit["logisticNu"]
        pk64 = pk.astype(np.float64)
        weights = 1.0 - 1.0 / (1.0 + np.exp(-logisticK * (-pk64 + peaksigThres))) ** logisticNu
    else:
        weights = pk
    lim = np.min([shapeImage[0] / 2.0, shapeImage[1] / 2.0] + ([] if maxShift is None else [N * maxShift]))
    rel = np.zeros([N, 2])
    weff = weights * accepted
    # the x and y solves are independent: y on a helper thread (the native
    # solver releases the GIL) while x runs here
    fy = _l1_pool().submit(l1_solve, A, b_y, weff, -lim, lim)
    rel[:, 1] = l1_solve(A, b_x, weff, -lim, lim)
    rel[:, 0] = fy.result()
    translations = -np.vstack((np.zeros([1, 2]), np.cumsum(rel, axis=0)))
    finish = functools.partial(_error_analysis, ed, A, rel, b_x, b_y, weights, accepted, N, unrav, M, translations,
                               shiftsTriMat_in)
    if defer_errors:
        return ed, translations, finish
    return finish()


def _error_analysis(ed, A, rel, b_x, b_y, weights, accepted, N, unrav, M, translations, shiftsTriMat_in):
    """The weighted error analysis of the drift solve (zorro.py:1484-1547),
    completing its errorDict."""
    weights = np.clip(weights, 1e-6, np.inf)
    errorXY = np.stack([A @ rel[:, 0] - b_y, A @ rel[:, 1] - b_x], axis=1)
    errorNorm = np.sqrt(errorXY[:, 0] ** 2 + errorXY[:, 1] ** 2)
    en = errorNorm[accepted]
    mean_e = np.sum(weights * en) / np.sum(weights)
    std_e = np.sqrt(np.sum(weights * en ** 2) / np.sum(weights) - mean_e ** 2)

    def unravel(v):
        out = np.zeros([N, N])
        out[unrav] = v
        return out

    errorUnraveled = unravel(errorNorm)
    acc = np.pad(unravel(accepted), ((0, 1), (1, 0)))
    ex = np.pad(unravel(np.abs(errorXY[:, 1])), ((0, 1), (1, 0))) * acc
    ey = np.pad(unravel(np.abs(errorXY[:, 0])), ((0, 1), (1, 0))) * acc
    wu = np.pad(unravel(weights), ((0, 1), (1, 0)))
    # per frame J: row J plus column J-1 (column -1 for J = 0, as Python
    # indexes it); the column sums run over contiguous copies of the columns,
    # so every sum adds the same numbers in the same order as np.sum of a row
    # or column slice
    prev = np.arange(N + 1) - 1

    def row_col(a):
        return a.sum(axis=1) + np.ascontiguousarray(a.T).sum(axis=1)[prev]

    with np.errstate(all="ignore"):
        den = row_col(wu)
        errorX = row_col(ex * wu) / den
        errorY = row_col(ey * wu) / den
    ed.update({"translations": translations, "relativeEst": rel,
               "acceptedEqns": accepted, "weights": weights, "errorXY": errorXY, "shiftsTriMat": shiftsTriMat_in,
               "errorX": errorX, "errorY": errorY, "errorUnraveled": errorUnraveled, "mean_errorNorm": mean_e,
               "std_errorNorm": std_e, "M": M, "Maccepted": M})
    return ed


def _sgn1(v):
    return -1.0 if v < 0.0 else 1.0


def brent_bounded(lo, hi, xatol, maxfun):
    """Bounded Brent minimisation (golden section and parabolic steps, the
    FMIN method of Forsythe, Malcolm and Moler behind scipy's
    minimize_scalar(method='bounded'), which locatePeak calls at
    zorro.py:1117) as a generator: it yields each abscissa, receives its
    function value through send(), and returns the best abscissa and the
    number of function values (StopIteration.value).  The steps are those
    of the peak kernel's device search, so that many planes can be searched
    in lock step with one batched evaluation per step."""
    sqrt_eps = math.sqrt(2.2e-16)
    golden = 0.5 * (3.0 - math.sqrt(5.0))
    a, b = lo, hi
    fulc = a + golden * (b - a)
    nfc = xf = fulc
    rat = e = 0.0
    x = xf
    fx = yield x
    num = 1
    ffulc = fnfc = fx
    xm = 0.5 * (a + b)
    tol1 = sqrt_eps * abs(xf) + xatol / 3.0
    tol2 = 2.0 * tol1
    while abs(xf - xm) > (tol2 - 0.5 * (b - a)):
        gstep = True
        if abs(e) > tol1:
            gstep = False
            r = (xf - nfc) * (fx - ffulc)
            q = (xf - fulc) * (fx - fnfc)
            p = (xf - fulc) * q - (xf - nfc) * r
            q = 2.0 * (q - r)
            if q > 0.0:
                p = -p
            q = abs(q)
            r = e
            e = rat
            if abs(p) < abs(0.5 * q * r) and p > q * (a - xf) and p < q * (b - xf):
                rat = (p + 0.0) / q
                x = xf + rat
                if (x - a) < tol2 or (b - x) < tol2:
                    rat = tol1 * _sgn1(xm - xf)
            else:
                gstep = True
        if gstep:
            e = (a - xf) if xf >= xm else (b - xf)
            rat = golden * e
        x = xf + _sgn1(rat) * max(abs(rat), tol1)
        fu = yield x
        num += 1
        if fu <= fx:
            if x >= xf:
                a = xf
            else:
                b = xf
            fulc, ffulc = nfc, fnfc
            nfc, fnfc = xf, fx
            xf, fx = x, fu
        else:
            if x < xf:
                a = x
            else:
                b = x
            if fu <= fnfc or nfc == xf:
                fulc, ffulc = nfc, fnfc
                nfc, fnfc = x, fu
            elif fu <= ffulc or fulc == xf or fulc == nfc:
                fulc, ffulc = x, fu
        xm = 0.5 * (a + b)
        tol1 = sqrt_eps * abs(xf) + xatol / 3.0
        tol2 = 2.0 * tol1
        if num >= maxfun:
            break
    return xf, num


def gaussian_taps(sigma, max_radius=64):
    """Taps of scipy.ndimage.gaussian_filter1d with truncate 4: radius
    int(4 sigma + 0.5), exp(-k^2 / (2 sigma^2)) normalised in double, as
    float32; one tap of 1 when sigma is 0 (the axis is not filtered)."""
    if not sigma > 1e-15:
        return np.ones(1, dtype=np.float32), 0
    r = min(int(4.0 * sigma + 0.5), max_radius)
    c = -0.5 / (sigma * sigma)
    g = [math.exp(c * k * k) for k in range(-r, r + 1)]
    s = 0.0
    for v in g:
        s += v
    return np.array([v / s for v in g], dtype=np.float32), r


def lanczos_kernel_1d(frac):
    """One axis of lanczosSubPixKernel(kernelShape=3, lobes=2), normalised.
    zorro_util.py:296-320 (the 2-D kernel is the outer product of the two
    axes, and its normalisation factors the same way)."""
    u = (2.0 / 3.0) * (np.arange(-1.5, 1.5) + 1.0 - frac)
    k = np.sinc(u * 2.0) * np.sinc(u)
    return k / np.sum(k)


SHIFT_DTYPE = np.dtype([("roll_y", "<i4"), ("roll_x", "<i4"), ("apply", "<i4"), ("ky", "<f4", 3), ("kx", "<f4", 3)])


def shift_table(translations, H, W, lanczos=True):
    """The zr_shift_t records of every frame at once (applyShifts,
    zorro.py:1734-1808 with lanczosIndexedShift, zorro_util.py:341-379): the
    integer roll (np.round) reduced to [0, H) x [0, W), and, with ``lanczos``,
    the two axes of the normalised Lanczos-2 kernel of the fractional
    remainder, skipped (apply = 0) when both remainders are close to zero.
    The same operations per frame as shift_params, on arrays."""
    t = np.asarray(translations).reshape(-1, 2)
    if not np.issubdtype(t.dtype, np.floating):
        t = t.astype(np.float64)  # float32 translations keep their precision, as in the reference
    out = np.zeros(len(t), dtype=SHIFT_DTYPE)
    it = np.round(t).astype(int)
    out["roll_y"] = np.mod(it[:, 0], H)
    out["roll_x"] = np.mod(it[:, 1], W)
    ident = np.array([0.0, 1.0, 0.0])
    if not lanczos:
        out["ky"] = ident
        out["kx"] = ident
        return out
    rem = np.remainder(t, 1)
    apply = ~(np.isclose(rem[:, 0], 0.0) & np.isclose(rem[:, 1], 0.0))
    base = np.arange(-1.5, 1.5) + 1.0

    def kern(frac):
        u = (2.0 / 3.0) * (base[None, :] - frac[:, None])
        k = np.sinc(u * 2.0) * np.sinc(u)
        return k / np.sum(k, axis=1, keepdims=True)
    out["apply"] = apply
    out["ky"] = np.where(apply[:, None], kern(rem[:, 0]), ident[None, :])
    out["kx"] = np.where(apply[:, None], kern(rem[:, 1]), ident[None, :])
    return out


def shift_params(translations):
    """Per-frame roll and sub-pixel kernel of applyShifts with
    shiftMethod='lanczos'.  zorro_util.py:341-379."""
    out = []
    for t in translations:
        it = np.round(t).astype(int)
        rem = np.remainder(t, 1)
        apply = not (np.isclose(rem[0], 0.0) and np.isclose(rem[1], 0.0))
        ky = lanczos_kernel_1d(rem[0]) if apply else np.array([0.0, 1.0, 0.0])
        kx = lanczos_kernel_1d(rem[1]) if apply else np.array([0.0, 1.0, 0.0])
        out.append((int(it[0]), int(it[1]), int(apply), ky, kx))
    return out


def frc_tiles(shape, trans, box=(512, 512), overlap=0.5, minCrop=5):
    """Tile offsets of tiledFRC.  zorro.py:2259-2289."""
    if overlap > 0.8:
        overlap = 0.8
    if trans is None or not np.any(trans):
        crop = np.array([minCrop] * 4, dtype=float)
    else:
        crop = np.array([np.maximum(np.ceil(trans[:, 0].max()), minCrop),
                         np.maximum(np.ceil(trans[:, 1].max()), minCrop),
                         -np.minimum(np.floor(trans[:, 0].min()), minCrop),
                         -np.minimum(np.floor(trans[:, 1].min()), minCrop)])
    tilesX = int(np.floor(float(shape[1] - crop[1] - crop[3] - box[1]) / box[1] / (1.0 - overlap)))
    tilesY = int(np.floor(float(shape[0] - crop[0] - crop[2] - box[0]) / box[0] / (1.0 - overlap)))
    offs = []
    for I in range(max(tilesY, 0)):
        for J in range(max(tilesX, 0)):
            offs.append(np.array([I * box[0] * (1.0 - overlap) + crop[0],
                                  J * box[1] * (1.0 - overlap) + crop[1]]).astype(int))
    return np.array(offs, dtype=np.int32).reshape(-1, 2), (tilesY, tilesX)


def dose_constants(m, shapePadded, pixelsize, voltage, doseFiltParam, imageSum_mean=None):
    """Dose-filter constants and per-frame cut-offs.  zorro.py:2375-2452
    (float64, the missing-dose term defined in both branches)."""
    A, B, Cc, order = (np.float32(doseFiltParam[i]) for i in (1, 2, 3, 4))
    if not voltage:
        raise ValueError("Accelerating voltage not set in advance for dose filtering")
    vs = np.float32(np.sqrt(voltage / 300.0))
    N, Mx = shapePadded
    invPSx = np.float32(1.0 / (Mx * (pixelsize * 10)))
    invPSy = np.float32(1.0 / (N * (pixelsize * 10)))
    dpf = (imageSum_mean / m) if doseFiltParam[0] is None else doseFiltParam[0]
    missing = dpf * np.float32(doseFiltParam[5])
    accum = np.zeros(m + 1)
    accum[1:] = np.cumsum(np.ones(m) * dpf)
    accum += missing
    qvect = np.arange(0, shapePadded[0] / 2) * np.sqrt(invPSx * invPSy)
    opti = np.zeros(int(shapePadded[0] / 2))
    with np.errstate(divide="ignore"):
        opti[1:] = np.float32(2.51284) * vs * (A * qvect[1:] ** B + Cc)
    opti[0] = opti[1] ** 2
    thresQ = np.empty(m)
    for J in range(m):
        idx = np.nonzero(np.abs(accum[J + 1] - opti) < np.abs(accum[J] - opti))[0]
        if idx.size == 0:
            raise ValueError("dose filter: no frequency where frame %d is closer to its optimal dose" % J)
        thresQ[J] = qvect[idx[-1]]
    return {"A": float(A), "B": float(B), "C": float(Cc), "order": float(order), "vs": float(vs),
            "invPSx": float(invPSx), "invPSy": float(invPSy), "dose_end": accum[1:].copy(), "thresQ": thresQ}


def hotpix_bins(sumMean, maxSigma):
    """Unit histogram bins of the unaligned sum.  zorro.py:2530-2533."""
    sumMean = np.float32(sumMean)
    poissonStd = np.sqrt(sumMean)
    edges = np.arange(np.floor(sumMean - maxSigma * poissonStd) - 0.5, np.ceil(sumMean + maxSigma * poissonStd) + 0.5, 1)
    return sumMean, poissonStd, edges


def _forward_points(x0, lb, ub, step, eps2):
    """The points of scipy's 2-point forward difference with absolute step
    ``step`` (approx_derivative: a step that does not change x taken
    relative to x, steps turned around or shortened to stay inside the
    bounds), and the realised steps."""
    pts, dx = [list(x0)], []
    for i, xi in enumerate(x0):
        h = step
        if (xi + h) - xi == 0.0:
            h = eps2 * (1.0 if xi >= 0 else -1.0) * max(1.0, abs(xi))
        lower_dist, upper_dist = xi - lb[i], ub[i] - xi
        xs = xi + h
        violated = xs < lb[i] or xs > ub[i]
        fitting = abs(h) <= max(lower_dist, upper_dist)
        if violated and fitting:
            h = -h
        elif not fitting:
            h = upper_dist if upper_dist >= lower_dist else -lower_dist
        x1 = list(x0)
        x1[i] = xi + h
        pts.append(x1)
        dx.append((xi + h) - xi)
    return pts, dx


def _value_and_gradient(f_rows, bounds, step=1e-8):
    """For minimize(..., jac=True): f(x) and the gradient L-BFGS-B estimates
    when no jac is given (the 2-point forward difference above), the same
    numbers (float64 operations on Python floats), with x and the forward
    points evaluated together in one call ``f_rows(points)`` -> values."""
    lb = [float(b[0]) for b in bounds]
    ub = [float(b[1]) for b in bounds]
    eps2 = float(np.finfo(np.float64).eps ** 0.5)

    def fg(x):
        x0 = [float(v) for v in np.asarray(x).ravel()]
        pts, dx = _forward_points(x0, lb, ub, step, eps2)
        v = f_rows(np.array(pts))
        return v[0], np.array([(v[1 + i] - v[0]) / dx[i] for i in range(len(dx))])
    return fg


def _setulb_loop(fg, x0, bounds, m=10, ftol=2.2204460492503131e-09, gtol=1e-5, maxfun=15000, maxiter=15000,
                 maxls=20):
    """The iterates of scipy.optimize.minimize(fg, x0, method='L-BFGS-B',
    jac=True, bounds=bounds) with its defaults: the same compiled step
    routine (scipy.optimize._lbfgsb.setulb) driven by the same loop as
    scipy's own driver, with f and g taken straight from ``fg`` (evaluated
    once per new x, as scipy's ScalarFunction does) instead of through its
    wrapper objects, whose Python overhead is most of the time of a small
    fit.  Returns x.  The call signature is that of scipy's C port of
    L-BFGS-B (scipy 1.15 and later); ``lbfgsb_minimize`` checks the result
    against scipy.optimize.minimize before using it."""
    from scipy.linalg.lapack import HAS_ILP64
    from scipy.optimize import _lbfgsb
    lb = np.array([float(b[0]) for b in bounds], dtype=np.float64)
    ub = np.array([float(b[1]) for b in bounds], dtype=np.float64)
    x = np.array(np.clip(np.asarray(x0).ravel(), lb, ub), dtype=np.float64)
    n = x.size
    it = np.int64 if HAS_ILP64 else np.int32
    nbd = np.full(n, 2, dtype=it)  # both bounds finite
    f = np.array(0.0, dtype=np.float64)
    g = np.zeros(n, dtype=np.float64)
    wa = np.zeros(2 * m * n + 5 * n + 11 * m * m + 8 * m, np.float64)
    iwa = np.zeros(3 * n, dtype=it)
    task = np.zeros(2, dtype=it)
    ln_task = np.zeros(2, dtype=it)
    lsave = np.zeros(4, dtype=it)
    isave = np.zeros(44, dtype=it)
    dsave = np.zeros(29, dtype=np.float64)
    factr = ftol / np.finfo(float).eps
    seen = None
    nfev = nit = 0
    while True:
        g = g.astype(np.float64)
        _lbfgsb.setulb(m, x, lb, ub, nbd, f, g, factr, gtol, wa, iwa, task, lsave, isave, dsave, maxls, ln_task)
        if task[0] == 3:  # f and g at x
            if seen is None or not np.array_equal(x, seen):
                seen = x.copy()
                fv, gv = fg(np.copy(seen))
                nfev += 1
            f, g = fv, np.atleast_1d(np.asarray(gv, dtype=np.float64))
        elif task[0] == 1:  # a new iterate
            nit += 1
            if nit >= maxiter:
                task[0], task[1] = 5, 504
            elif nfev > maxfun:
                task[0], task[1] = 5, 502
        else:
            break
    return x


_SETULB_OK = None  # None: not checked yet; then True or False


def _setulb_usable():
    """Whether _setulb_loop reproduces scipy.optimize.minimize here: both
    run once on a fixed bounded fit (a normal CDF fitted to a seeded
    histogram, as the hot-pixel fit does); any difference or error keeps
    scipy.optimize.minimize."""
    global _SETULB_OK
    if _SETULB_OK is None:
        try:
            rng = np.random.default_rng(2024)
            vals = rng.poisson(20.0, size=200000).astype(np.float64)
            edges = np.arange(np.floor(20.0 - 7 * np.sqrt(20.0)) - 0.5, np.ceil(20.0 + 7 * np.sqrt(20.0)) + 0.5, 1)
            hist = np.histogram(vals, bins=edges)[0].astype(np.float64)
            counts = edges[:-1] + 0.5
            cdf = np.cumsum(hist) / hist.sum()

            def rows(P):
                return np.sum(np.abs(cdf[None, :] - scipy.special.ndtr((counts[None, :] - P[:, 0:1]) / P[:, 1:2])),
                              axis=1)

            s = np.sqrt(20.0)
            bounds = ((20.0 - 0.5 * s, 20.0 + 0.5 * s), (0.7 * s, 1.3 * s))
            fg = _value_and_gradient(rows, bounds)
            ref = scipy.optimize.minimize(fg, (19.3, 1.1 * s), method="L-BFGS-B", bounds=bounds, jac=True).x
            _SETULB_OK = bool(np.array_equal(_setulb_loop(fg, (19.3, 1.1 * s), bounds), ref))
        except Exception:
            _SETULB_OK = False
    return _SETULB_OK


def lbfgsb_minimize(fg, x0, bounds):
    """x of scipy.optimize.minimize(fg, x0, method='L-BFGS-B', jac=True,
    bounds=bounds): by the direct loop where it gives scipy's result, else
    by scipy.optimize.minimize itself."""
    if _setulb_usable():
        return _setulb_loop(fg, x0, bounds)
    return scipy.optimize.minimize(fg, x0, method="L-BFGS-B", bounds=bounds, jac=True).x


def hotpix_fit(hist, edges, sumMean, poissonStd, hotpixInfo):
    """Normal-CDF fit and the outlier cut-offs.  zorro.py:2535-2592.  An empty
    line fit falls back to the configured default, as it did when
    np.linalg.lstsq raised on empty systems."""
    hist = np.asarray(hist, dtype=np.float64)
    counts = np.asarray(edges[:-1], dtype=np.float64).copy()
    counts += 0.5 * (counts[1] - counts[0])
    cdf = np.cumsum(hist)
    cdf /= cdf[-1]

    def err_rows(P):
        # sum |cdf - norm.cdf(counts, loc, scale)| (zorro.py:2553) for every
        # row (loc, scale) of P; norm.cdf evaluates ndtr((counts - loc) /
        # scale), and each row sums as a 1-D array would
        z = (counts[None, :] - P[:, 0:1]) / P[:, 1:2]
        return np.sum(np.abs(cdf[None, :] - scipy.special.ndtr(z)), axis=1)

    bounds = ((sumMean - 0.5 * poissonStd, sumMean + 0.5 * poissonStd), (0.7 * poissonStd, 1.3 * poissonStd))
    bx = lbfgsb_minimize(_value_and_gradient(err_rows, bounds), (sumMean, poissonStd), bounds)
    with np.errstate(all="ignore"):
        sig_cdf = np.sqrt(2) * scipy.special.erfinv(2.0 * cdf - 1)
    normal = (counts - bx[0]) / bx[1]
    e = normal - sig_cdf
    keep = ~np.isinf(e)
    e = e[keep]
    nk = normal[keep]
    info = {}
    cl = np.float32(hotpixInfo["cutoffLower"])
    cu = np.float32(hotpixInfo["cutoffUpper"])
    try:
        li = np.nonzero(e > -0.5)[0][0]
        if li > 0:
            f = np.linalg.lstsq(np.stack([nk[:li], np.ones(li)], axis=1), e[:li], rcond=None)[0]
            cl = np.float32(-f[1] / f[0])
            info["cutoffLower"] = float(cl)
    except IndexError:
        pass
    try:
        ui = np.nonzero(e < 0.5)[0][-1]
        if ui < len(nk):
            f = np.linalg.lstsq(np.stack([nk[ui:], np.ones(len(nk) - ui)], axis=1), e[ui:], rcond=None)[0]
            cu = np.float32(-f[1] / f[0])
            info["cutoffUpper"] = float(cu)
    except IndexError:
        pass
    return bx[0], bx[1], cl, cu, info


def psf_kernel(psf="K2"):
    """3x3 detector PSF of hotpixFilter.  zorro.py:2511-2519."""
    p1 = 0.173235968 if psf == "K2" else 1.0
    k = np.array([[p1 * p1, p1, p1 * p1], [p1, 0.0, p1], [p1 * p1, p1, p1 * p1]])
    return k / np.sum(k)

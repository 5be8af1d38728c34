"""CPU restatement of Zorro's movie-registration hot path (the oracle).

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may use this module, and only as the checker
or as the timed CPU baseline; the CUDA product path never calls it.

Every function restates one step of ``ImageRegistrator.alignImageStack``
(LBEM-CH/zorro ``zorro/zorro.py``) in NumPy/SciPy, with the reference's line
numbers in its docstring.  The arithmetic follows the reference literally,
quirks included (the suppressOrigin stencil, the Denom clip, ``np.remainder``
sub-pixel shifts, the ``abs()`` of the dose-filtered sum).  ``fp64=True`` runs
in float64/complex128 (the accuracy oracle); ``fp64=False`` runs in the
reference's native float32/complex64 (the CPU baseline).

Parity: pinned against fixtures produced by running the unmodified reference
(``oracle/ref_harness.py`` via ``tests/golden/make_golden.py``).  Two choices
are fixed where the reference is stochastic (its shift solve and logistic fit
use unseeded ``scipy.optimize.basinhopping``): the shift solve returns the
exact weighted-L1 optimum (linear programme, HiGHS) and the logistic fit is
the deterministic Nelder-Mead minimisation of ``logistic_fit_deterministic``
on the same objective, start point and bounds.
"""
from __future__ import annotations

import time

import numpy as np
import scipy.fft
import scipy.ndimage
import scipy.optimize
import scipy.special
import scipy.stats

LOGISTIC_SEED = 1234


class Dtypes:
    def __init__(self, fp64=True, workers=1):
        self.c = np.complex128 if fp64 else np.complex64
        self.f = np.float64 if fp64 else np.float32
        self.workers = workers

    def fft2(self, a):
        return scipy.fft.fft2(a.astype(self.c, copy=False), workers=self.workers)

    def ifft2(self, a):
        """The inverse as the reference's FFTW plans run it (execute():
        unscaled; its normConst factors account for that)."""
        return scipy.fft.ifft2(a, norm="forward", workers=self.workers)


# --------------------------------------------------------------------------
# triangle of pairs, padding, Fourier crop
# --------------------------------------------------------------------------

def tri_indices(N, triMode="diag", diagWidth=5, diagStart=0):
    """Boolean [N,N] matrix of correlated pairs.  zorro.py:558-579."""
    xmesh, ymesh = np.meshgrid(np.arange(N), np.arange(N))
    trimesh = xmesh - ymesh
    if triMode == "first":
        t = np.ones([1, N], dtype=bool)
        t[0, 0] = False
        return t
    if triMode == "diag":
        if diagWidth is None or diagWidth < 0:
            diagWidth = N
        return (trimesh <= diagWidth + diagStart) * (trimesh > diagStart)
    if triMode in ("autocorr", "refine"):
        return trimesh == 0
    return trimesh >= 1


def bin_stack(images, shapeBinned, dt):
    """Fourier binning, binStack(binKernel='fourier').  zorro.py:1826-1904:
    per frame the full FFT, the four corners of Hb/2 x Wb/2 kept, times
    1/(Hb Wb), the unscaled inverse, its real part as float32."""
    b0, b1 = int(shapeBinned[0]) // 2, int(shapeBinned[1]) // 2
    out = np.zeros([images.shape[0], int(shapeBinned[0]), int(shapeBinned[1])], dtype="float32")
    normConst = 1.0 / (shapeBinned[0] * shapeBinned[1])
    for J in range(images.shape[0]):
        F = dt.fft2(images[J].astype(dt.c))
        B = np.zeros([int(shapeBinned[0]), int(shapeBinned[1])], dtype=dt.c)
        B[:b0, :b1] = F[:b0, :b1]
        B[:b0, -b1:] = F[:b0, -b1:]
        B[-b0:, :b1] = F[-b0:, :b1]
        B[-b0:, -b1:] = F[-b0:, -b1:]
        B *= normConst
        out[J] = np.real(dt.ifft2(B))
    return out


def pad_stack(images, shapePadded):
    """Zero-pad at the top-left and build the [1,P,P] mask.  zorro.py:1908-1958."""
    m, H, W = images.shape
    out = np.zeros([m, shapePadded[0], shapePadded[1]], dtype=images.dtype)
    out[:, :H, :W] = images
    mask = np.zeros([1, shapePadded[0], shapePadded[1]], dtype=bool)
    mask[0, :H, :W] = True
    return out, mask


def fourier_crop(F, shapeCropped):
    """Keep the four corners of a spectrum.  zorro.py:901-904 (FFTCrop)."""
    sC2 = (np.asarray(shapeCropped) // 2).astype(int)
    out = np.empty(shapeCropped, dtype=F.dtype)
    out[0:sC2[0], 0:sC2[1]] = F[0:sC2[0], 0:sC2[1]]
    out[0:sC2[0], -sC2[1]:] = F[0:sC2[0], -sC2[1]:]
    out[-sC2[0]:, 0:sC2[1]] = F[-sC2[0]:, 0:sC2[1]]
    out[-sC2[0]:, -sC2[1]:] = F[-sC2[0]:, -sC2[1]:]
    return out


def shape_cropped(fouCrop):
    """zorro.py:607 (force even)."""
    return 2 * np.floor(np.array(fouCrop) / 2.0).astype(int)


def norm_const2(shapeCropped):
    """zorro.py:634 -- rounded to float32 as in the reference."""
    return float(np.float32(1.0 / (np.float64(shapeCropped[0]) * np.float64(shapeCropped[1])) ** 2.0))


# --------------------------------------------------------------------------
# spectra and the masked normalised cross-correlation
# --------------------------------------------------------------------------

def mask_spectrum(mask, sC, dt):
    """Mask FFT + FFTCrop and maskProduct.  zorro.py:814-835."""
    GM = fourier_crop(dt.fft2(mask[0].astype(dt.c)), sC)
    nc2 = norm_const2(sC)
    MP = nc2 * np.real(dt.ifft2(np.conj(GM) * GM))
    return GM, MP.astype(dt.f, copy=False)


def frame_spectra(frame_padded, mask, sC, dt):
    """FFT(m*I) and FFT((m*I)^2), both Fourier-cropped.  zorro.py:875-914."""
    tempReal = (mask[0] * frame_padded).astype(dt.c)
    G = fourier_crop(dt.fft2(tempReal), sC)
    S = fourier_crop(dt.fft2(tempReal * tempReal), sC)
    return G, S


def mnxc2(GI, SI, GJ, SJ, GM, MP, nc2, maxShift, suppressOrigin=True, dt=None):
    """Padfield masked normalised cross-correlation of template I with base J,
    cropped to the +/-maxShift window.  zorro.py:1014-1097.

    Returns (C window [2*maxShift]^2, origin value C[0,0])."""
    tGI = np.conj(GI)
    CTM = np.real(dt.ifft2(GM * tGI)) * nc2
    CBM = np.real(dt.ifft2(np.conj(GM) * GJ)) * nc2
    tc = dt.ifft2(GM * np.conj(SI))
    tc2 = dt.ifft2(np.conj(GM) * SJ)
    with np.errstate(all="ignore"):
        Denom = np.sqrt((np.real(tc2) * nc2 - np.real(CBM * (CBM / MP)))
                        * (np.real(tc) * nc2 - np.real(CTM * (CTM / MP))))
        Denom = np.clip(Denom, 1, np.inf)
        tc = dt.ifft2(GJ * tGI)
        C = (np.real(tc) * nc2 - np.real(CTM * CBM / MP)) / Denom
    origin = C[0, 0]
    if suppressOrigin:
        # literal stencil of zorro.py:1082-1083 ([-1,0] and [-1,1] twice)
        C[0, 0] = 0.125 * (C[1, 0] + C[0, 1] + C[-1, 0] + C[-1, 0] +
                           C[1, 1] + C[-1, 1] + C[-1, 1] + C[-1, -1])
    C = np.fft.ifftshift(C)
    if maxShift is not None:
        c2 = (np.array(C.shape) / 2.0).astype(int)
        C = C[c2[0] - maxShift:c2[0] + maxShift, c2[1] - maxShift:c2[1] + maxShift]
    return C.astype(dt.f, copy=False), origin


def max_shift_mask(maxShift):
    """zorro.py:846-851."""
    xmesh, ymesh = np.meshgrid(np.arange(-maxShift, maxShift), np.arange(-maxShift, maxShift))
    return (xmesh * xmesh + ymesh * ymesh) < maxShift ** 2.0


def opti_sigma(C):
    """Bmode 'opti': bounded Brent search for the Gaussian sigma that
    maximises peak contrast.  zorro.py:1105-1121."""
    def inversePeakContrast(Bsigma):
        Cf = scipy.ndimage.gaussian_filter(C, Bsigma)
        return np.std(Cf) / (np.max(Cf) - np.mean(Cf))
    res = scipy.optimize.minimize_scalar(inversePeakContrast, bounds=[0.0, 7.0], method="bounded",
                                         options={"maxiter": 15, "xatol": 0.01})
    return float(res.x), scipy.ndimage.gaussian_filter(C, res.x)


def locate_peak(C, mask_maxShift, subPixReg=16, Bmode="opti", Brad=512, shapePadded=None, dt=None, roll=None):
    """Peak position with Fourier-interpolated sub-pixel refinement.
    zorro.py:1099-1231.  With ``roll`` (preShift, zorro.py:1148-1162) the
    search mask is np.roll-ed by (roll[0], roll[1]) first.

    Returns dict(shift[2], corr, peaksig, sigma, C_filt)."""
    sigma = None
    if Bmode == "opti":
        sigma, C_filt = opti_sigma(C)
    elif Brad and Bmode in ("conv", "convolution"):
        Bsigma = np.asarray(shapePadded) / (np.sqrt(2) * np.pi * Brad)
        C_filt = scipy.ndimage.gaussian_filter(C, Bsigma)
    else:
        C_filt = C
    subR = 8
    if mask_maxShift is not None and roll is not None:
        mask_maxShift = np.roll(np.roll(mask_maxShift, int(roll[0]), axis=0), int(roll[1]), axis=1)
    if mask_maxShift is not None:
        C_masked = C_filt * mask_maxShift
        cmaxpos = np.unravel_index(np.argmax(C_masked), C_filt.shape)
        peaksig = (C_masked[cmaxpos] - np.mean(C_filt[mask_maxShift])) / np.std(C_filt[mask_maxShift])
    else:
        cmaxpos = np.unravel_index(np.argmax(C_filt), C_filt.shape)
        peaksig = np.nan
    shape = np.array(C.shape)
    if subPixReg > 1.0:
        Csub = C_filt[cmaxpos[0] - subR:cmaxpos[0] + subR, cmaxpos[1] - subR:cmaxpos[1] + subR]
        if Csub.shape[0] == 2 * subR and Csub.shape[1] == 2 * subR:
            CsubFFT = dt.fft2(Csub.astype(dt.c))
            npad = (subPixReg - 1) * subR
            Cpad = np.zeros([subPixReg * subR * 2] * 2, dtype=dt.c)
            Cpad.real = np.pad(np.fft.fftshift(CsubFFT.real), ((npad,),), mode="constant")
            Cpad.imag = np.pad(np.fft.fftshift(CsubFFT.imag), ((npad,),), mode="constant")
            Cpad = np.fft.ifftshift(Cpad)
            over = np.abs(dt.ifft2(Cpad))
            smax = np.unravel_index(np.argmax(over), over.shape)
            round_pos = np.array(cmaxpos) - shape / 2.0
            remainder = (np.array(smax) - np.array(over.shape) / 2.0 + np.sign(round_pos)) / subPixReg
            shift = round_pos + remainder
            corr = over[smax] / (subR * 2.0) ** 2.0
        else:
            shift = np.array(cmaxpos) - shape / 2.0
            corr = C[cmaxpos]
    else:
        shift = np.array(cmaxpos) - shape / 2.0
        corr = C[cmaxpos]
    return {"shift": shift, "corr": float(corr), "peaksig": float(peaksig), "sigma": sigma,
            "C_filt": C_filt, "cmaxpos": cmaxpos}


def preshift_mask(sC, maxShift):
    """The search mask of preShift: the whole cropped grid, radius maxShift
    about its centre.  zorro.py:841-851 (preShift branch)."""
    c2 = (np.array(sC) / 2.0).astype(int)
    xmesh, ymesh = np.meshgrid(np.arange(-c2[0], c2[0]), np.arange(-c2[1], c2[1]))
    return (xmesh * xmesh + ymesh * ymesh) < maxShift ** 2.0


def xcorr_tri(images_padded, mask, *, shapePadded, fouCrop, triMode="diag", diagWidth=5, diagStart=0,
              maxShift=100, subPixReg=16, Bmode="opti", Brad=512, suppressOrigin=True, dt=None,
              capture=None, pairs_limit=None, preShift=False, peaksigThres=6.0, autoMax=10):
    """All-pairs registration.  zorro.py:773-1011 (single mask).  triMode
    'refine' (zorro.py:934-954) correlates each frame I < N-1 with the
    template conj(sum_n G_n - G_I) / N (and likewise for the squared
    spectra), filling the diagonal.  With ``preShift`` (zorro.py:1089-1092,
    1148-1162) the correlation planes are not cropped and the maxShift disc
    is rolled by the rounded shift of the previous pair of the row,
    shiftsTriMat[I, J-1] ('refine': shiftsTriMat[I-1, I-1]), as measured so
    far in cropped pixels.  triMode 'auto' stops a row after the first pair
    whose peak significance is <= peaksigThres or whose J - I >= autoMax
    (zorro.py:995-997).  Returns (shiftsTriMat, corrTriMat, peaksigTriMat,
    originTriMat)."""
    N = images_padded.shape[0]
    tri = tri_indices(N, triMode, diagWidth, diagStart)
    if np.any(fouCrop):
        sC = shape_cropped(fouCrop)
    else:
        sC = np.array(images_padded.shape[1:])
    nc2 = norm_const2(sC)
    GM, MP = mask_spectrum(mask, sC, dt)
    pre = bool(preShift) and bool(maxShift)
    mmask = (preshift_mask(sC, maxShift) if pre else max_shift_mask(maxShift)) if maxShift else None
    crop = None if pre else maxShift
    G = [None] * N
    S = [None] * N
    for I in range(N):
        G[I], S[I] = frame_spectra(images_padded[I], mask, sC, dt)
    shifts = np.zeros([N, N, 2], dtype=dt.f)
    corr = np.zeros([N, N], dtype=dt.f)
    peaksig = np.zeros([N, N], dtype=dt.f)
    origin = np.zeros([N, N], dtype=dt.f)
    done = 0
    if triMode == "refine":
        sumG = np.sum(np.stack(G), axis=0)
        sumS = np.sum(np.stack(S), axis=0)
        for I in range(N - 1):
            # mnxc2 conjugates its template argument: conj((sum - G_I) / N)
            # equals the reference's conj(sum - G_I) / N exactly
            C, o = mnxc2((sumG - G[I]) / N, (sumS - S[I]) / N, G[I], S[I], GM, MP, nc2, crop, suppressOrigin,
                         dt)
            origin[I, I] = o
            roll = np.round(shifts[I - 1, I - 1]).astype(int) if pre else None
            r = locate_peak(C, mmask, subPixReg, Bmode, Brad, shapePadded, dt, roll=roll)
            shifts[I, I, :] = r["shift"]
            corr[I, I] = r["corr"]
            peaksig[I, I] = r["peaksig"]
            if capture is not None:
                capture[(int(I), int(I))] = {"C": C, "sigma": r["sigma"], "C_filt": r["C_filt"]}
    pair_rows = [] if triMode == "refine" else np.unique(np.argwhere(np.sum(tri, axis=1) > 0))
    for I in pair_rows:
        for J in np.unique(np.argwhere(tri[I, :])):
            C, o = mnxc2(G[I], S[I], G[J], S[J], GM, MP, nc2, crop, suppressOrigin, dt)
            origin[I, J] = o
            roll = np.round(shifts[I, J - 1]).astype(int) if pre else None
            r = locate_peak(C, mmask, subPixReg, Bmode, Brad, shapePadded, dt, roll=roll)
            shifts[I, J, :] = r["shift"]
            corr[I, J] = r["corr"]
            peaksig[I, J] = r["peaksig"]
            if capture is not None:
                capture[(int(I), int(J))] = {"C": C, "sigma": r["sigma"], "C_filt": r["C_filt"]}
            done += 1
            if pairs_limit is not None and done >= pairs_limit:
                break
            if triMode == "auto" and (peaksig[I, J] <= peaksigThres or J - I >= autoMax):
                break
        if pairs_limit is not None and done >= pairs_limit:
            break
    if np.any(fouCrop):
        shifts[:, :, 0] *= shapePadded[0] / sC[0]
        shifts[:, :, 1] *= shapePadded[1] / sC[1]
    return shifts, corr, peaksig, origin


# --------------------------------------------------------------------------
# shift solve
# --------------------------------------------------------------------------

def weighted_l1_exact(A, b, w, bounds):
    """argmin sum(w*|A x - b|) in a box (the objective of
    zorro_util.py:849-851), exactly.  Solved as the dual linear programme
    max b.y s.t. A^T y = 0, |y| <= w (HiGHS), whose equality multipliers are
    the primal optimum; when that point leaves the box the bounded primal LP
    is solved instead."""
    A = np.asarray(A, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    w = np.asarray(w, dtype=np.float64)
    m, n = A.shape
    bnd = np.asarray(bounds, dtype=np.float64)
    res = scipy.optimize.linprog(-b, A_eq=A.T, b_eq=np.zeros(n), bounds=list(zip(-w, w)), method="highs")
    if res.success:
        x = -res.eqlin.marginals
        if np.all(x >= bnd[:, 0]) and np.all(x <= bnd[:, 1]):
            return x
    c = np.concatenate([np.zeros(n), w])
    I = np.eye(m)
    A_ub = np.block([[A, -I], [-A, -I]])
    b_ub = np.concatenate([b, -b])
    bnds = [tuple(map(float, bb)) for bb in bnd] + [(0.0, None)] * m
    res = scipy.optimize.linprog(c, A_ub=A_ub, b_ub=b_ub, bounds=bnds, method="highs")
    if not res.success:
        raise RuntimeError("weighted L1 LP failed: " + str(res.message))
    return res.x[:n]


def min_logistic(x, hSigma, cdf):
    """zorro_util.py:862-863."""
    return np.float32(np.sum(np.abs(cdf - (1.0 - 1.0 / (1.0 + np.exp(-x[1] * (-hSigma + x[0])))
                                           ** np.float64(x[2])))))


def _logistic_cdf_error64(x, hSigma, cdf):
    """min_logistic without its final float32 cast (zorro_util.py:862-863)."""
    with np.errstate(over="ignore"):
        return np.sum(np.abs(cdf - (1.0 - 1.0 / (1.0 + np.exp(-x[1] * (-hSigma + x[0]))) ** x[2])))


def logistic_fit_deterministic(hSigma, cdf, lo, hi, mean):
    """A deterministic minimiser of the reference's logistic-CDF error within
    its bounds (zorro.py:2000-2008): Nelder-Mead from the reference's start
    point (mean, 5, 1), to tight tolerances.  The reference's unseeded
    basinhopping returns a different point every run and jumps between
    near-equal minima under 1e-9 perturbations of its input; this minimiser
    repeats and moves continuously with its input."""
    bounds = ((lo, hi), (0.1, 20.0), (0.05, 5.0))
    with np.errstate(over="ignore"):
        r = scipy.optimize.minimize(_logistic_cdf_error64, (mean, 5.0, 1.0), args=(hSigma, cdf), method="Nelder-Mead",
                                    bounds=bounds, options={"xatol": 1e-10, "fatol": 1e-14, "maxiter": 4000,
                                                            "maxfev": 8000})
    return r.x


def cdf_logistic_curve(peaksigTriMat, seed=LOGISTIC_SEED):
    """Fit a logistic to the CDF of peak significances.  zorro.py:1981-2022
    (histogram and objective as the reference; the minimiser is
    logistic_fit_deterministic)."""
    peaksigs = peaksigTriMat[peaksigTriMat > 0.0]
    bins = int(peaksigs.size / 7.0)
    pdfPeaks, hSigma = np.histogram(peaksigs, bins=bins)
    hSigma = hSigma[:-1]
    pdfPeaks = pdfPeaks.astype("float32")
    cdfPeaks = np.cumsum(pdfPeaks)
    cdfPeaks /= cdfPeaks[-1]
    x = logistic_fit_deterministic(hSigma, cdfPeaks, np.min(peaksigs), np.max(peaksigs), np.mean(peaksigs))
    return {"peaksigThres": x[0], "logisticK": x[1], "logisticNu": x[2],
            "pdfPeaks": pdfPeaks, "cdfPeaks": cdfPeaks, "hSigma": hSigma}


def solver_matrix(triIndices):
    """Equation matrix of the relative-shift solve.  zorro.py:1292-1311."""
    N = triIndices.shape[0]
    last_col = np.zeros(N, dtype=int)
    M = 0
    for I in range(N):
        if triIndices[I, :].any():
            last_col[I] = np.argwhere(triIndices[I, :])[-1][0] + 1
            M += last_col[I] - I
    A = np.zeros([int(M), N])
    pos = 0
    for I in range(N):
        rv = np.rot90(triIndices[I:last_col[I], I:last_col[I]], k=2)
        A[pos:pos + rv.shape[0], I:I + rv.shape[1]] = rv
        pos += rv.shape[0]
    return A


def shifts_solver(shiftsTriMat_in, corrTriMat_in, peaksigTriMat_in, *, shapeImage, maxShift,
                  weightMode="autologistic", peaksigThres=6.0, logisticK=5.0, logisticNu=0.15,
                  seed=LOGISTIC_SEED):
    """Weighted-L1 solve for the per-frame drift.  zorro.py:1260-1567."""
    shiftsTriMat = shiftsTriMat_in[:-1, 1:, :]
    corrTriMat = corrTriMat_in[:-1, 1:]
    peaksigTriMat = peaksigTriMat_in[:-1, 1:]
    triIndices = corrTriMat.astype(bool)
    ed = {"corrTriMat": corrTriMat_in, "peaksigTriMat": peaksigTriMat_in}
    N = shiftsTriMat_in.shape[0] - 1
    A = solver_matrix(triIndices)
    M = A.shape[0]
    vectorIndices = np.arange(0, triIndices.size)[np.ravel(triIndices)]
    unravelIndices = np.unravel_index(vectorIndices, [N, N])
    b_x = np.ravel(shiftsTriMat[triIndices, 1])
    b_y = np.ravel(shiftsTriMat[triIndices, 0])
    acceptedEqns = np.ones_like(b_x, dtype=bool)
    Maccepted = M
    ps = np.ravel(peaksigTriMat[triIndices])
    if weightMode is None or weightMode == "corr":
        weights = ps
    elif weightMode == "unweighted":
        weights = np.ones_like(ps)
    elif weightMode in ("norm", "normalized"):
        weights = (ps - ps.min()) / (ps.max() - ps.min())
    elif weightMode in ("autologistic", "logistic"):
        if weightMode == "autologistic":
            fit = cdf_logistic_curve(peaksigTriMat_in, seed)
            ed.update(fit)
            peaksigThres, logisticK, logisticNu = fit["peaksigThres"], fit["logisticK"], fit["logisticNu"]
        pk = ps.astype("float64")
        weights = 1.0 - 1.0 / (1.0 + np.exp(-logisticK * (-pk + peaksigThres))) ** logisticNu
    else:
        weights = ps
    bounds = np.ones([N, 2])
    bounds[:, 0] = -1.0
    if maxShift is None:
        bounds *= np.min([shapeImage[0] / 2.0, shapeImage[1] / 2.0])
    else:
        bounds *= np.min([shapeImage[0] / 2.0, shapeImage[1] / 2.0, N * maxShift])
    rel = np.zeros([N, 2])
    w_eff = weights * acceptedEqns
    rel[:, 1] = weighted_l1_exact(A, b_x, w_eff, bounds)
    rel[:, 0] = weighted_l1_exact(A, b_y, w_eff, bounds)
    # weighted error analysis, zorro.py:1484-1547
    weights = np.clip(weights, 1e-6, np.inf)
    errorXY = np.zeros([M, 2])
    errorXY[:, 1] = A @ rel[:, 1] - b_x
    errorXY[:, 0] = A @ rel[:, 0] - b_y
    errorNorm = np.sqrt(errorXY[:, 0] ** 2 + errorXY[:, 1] ** 2)
    aen = errorNorm[acceptedEqns]
    mean_e = np.sum(weights * aen) / np.sum(weights)
    std_e = np.sqrt(np.sum(weights * aen ** 2) / np.sum(weights) - mean_e ** 2)
    errorUnraveled = np.zeros([N, N])
    errorXun = np.zeros([N, N])
    errorYun = np.zeros([N, N])
    weightsUn = np.zeros([N, N])
    errorUnraveled[unravelIndices] = errorNorm
    weightsUn[unravelIndices] = weights
    errorXun[unravelIndices] = np.abs(errorXY[:, 1])
    errorYun[unravelIndices] = np.abs(errorXY[:, 0])
    accUn = np.zeros([N, N])
    accUn[unravelIndices] = acceptedEqns
    accUn = np.pad(accUn, ((0, 1), (1, 0)))
    errorXun = np.pad(errorXun, ((0, 1), (1, 0))) * accUn
    errorYun = np.pad(errorYun, ((0, 1), (1, 0))) * accUn
    weightsUn = np.pad(weightsUn, ((0, 1), (1, 0)))
    errorX = np.zeros(N + 1)
    errorY = np.zeros(N + 1)
    with np.errstate(all="ignore"):
        for J in range(N + 1):
            den = np.sum(weightsUn[J, :]) + np.sum(weightsUn[:, J - 1])
            errorX[J] = (np.sum(errorXun[J, :] * weightsUn[J, :]) + np.sum(errorXun[:, J - 1] * weightsUn[:, J - 1])) / den
            errorY[J] = (np.sum(errorYun[J, :] * weightsUn[J, :]) + np.sum(errorYun[:, J - 1] * weightsUn[:, J - 1])) / den
    ed.update({"translations": -np.vstack((np.zeros([1, 2]), np.cumsum(rel, axis=0))),
               "relativeEst": rel, "acceptedEqns": acceptedEqns, "weights": weights, "errorXY": errorXY,
               "shiftsTriMat": shiftsTriMat_in, "errorX": errorX, "errorY": errorY,
               "errorUnraveled": errorUnraveled, "mean_errorNorm": mean_e, "std_errorNorm": std_e,
               "M": M, "Maccepted": Maccepted})
    return ed


# --------------------------------------------------------------------------
# shift and sum, FRC, dose filter, hot pixels
# --------------------------------------------------------------------------

def lanczos_kernel(subPixShift, kernelShape=3, lobes=None):
    """zorro_util.py:296-320."""
    ks = np.array([kernelShape, kernelShape], dtype=int)
    if lobes is None:
        lobes = (ks[0] + 1) / 2
    x = (2.0 / ks[1]) * (np.arange(-ks[1] / 2, ks[1] / 2) + 1.0 - subPixShift[1])
    y = (2.0 / ks[0]) * (np.arange(-ks[1] / 2, ks[0] / 2) + 1.0 - subPixShift[0])
    xm, ym = np.meshgrid(x, y)
    k = np.sinc(xm * lobes) * np.sinc(xm) * np.sinc(ym * lobes) * np.sinc(ym)
    return k / np.sum(k)


def apply_shifts(images, translations, originMode="centroid", shiftMethod="lanczos", subPixReg=16, shapePadded=None,
                 dt=None):
    """Shift every frame and sum.  zorro.py:1734-1808 with
    zorro_util.py:341-379 (lanczosIndexedShift).  ``images`` is modified in
    place; returns (translations_applied, imageSum).  (shiftMethod 'fourier'
    never gets here: see align_image_stack.)"""
    # the reference keeps the translations' dtype (float32 after 'refine',
    # zorro.py:1643), and with it the precision of the centroid
    t = np.array(translations, copy=True)
    if not np.issubdtype(t.dtype, np.floating):
        t = t.astype(np.float64)
    if originMode == "centroid":
        t -= np.mean(t, axis=0)
    if subPixReg > 1.0 and shiftMethod == "lanczos":
        for J in range(images.shape[0]):
            it = np.round(t[J]).astype(int)
            images[J] = np.roll(np.roll(images[J], it[0], axis=0), it[1], axis=1)
            rem = np.remainder(t[J], 1)
            if not (np.isclose(rem[0], 0.0) and np.isclose(rem[1], 0.0)):
                k = lanczos_kernel(rem, 3, None)
                images[J] = scipy.ndimage.convolve(images[J], k, mode="reflect")
    else:
        it = np.round(t).astype(int)
        for J in range(images.shape[0]):
            images[J] = np.roll(np.roll(images[J], it[J, 0], axis=0), it[J, 1], axis=1)
    return t, np.sum(images, axis=0)


def apodization_hann(shape):
    """'hann' window of zorro_util.py:62-120 (radius = shape/2)."""
    shape = np.asarray(shape)
    radius = shape / 2.0
    xm, ym = np.meshgrid(np.arange(-shape[1] / 2, shape[1] / 2), np.arange(-shape[0] / 2, shape[0] / 2))
    rr = (xm / radius[1]) ** 2.0 + (ym / radius[0]) ** 2.0
    return (rr <= 1.0).astype(float) * 0.5 * (1.0 + np.cos(np.pi * np.sqrt(rr)))


def rotmean(mage):
    """Rotational mean with bilinear ring weights.  zorro_util.py:147-224."""
    if mage.shape[0] % 2 or mage.shape[1] % 2:
        raise ValueError("rotmean restatement expects even shapes")
    N = mage.shape[1] // 2
    M = mage.shape[0] // 2
    rmax = int(np.ceil(np.sqrt(N ** 2 + M ** 2)) + 1)
    xm, ym = np.meshgrid(np.arange(-N, N), np.arange(-M, M))
    r = np.sqrt(xm ** 2 + ym ** 2)
    rf = np.floor(r)
    remain = (r - rf).ravel()
    rf = rf.ravel().astype(int)
    rc = rf + 1
    weights = np.bincount(rc, remain) + np.bincount(rf, 1.0 - remain, minlength=rmax)
    m = mage.ravel()
    rmean = np.bincount(rc, m * remain) + np.bincount(rf, m * (1.0 - remain), minlength=rmax)
    return rmean / weights


def frc_crop_limits(trans, minCrop=5):
    """zorro.py:2266-2274."""
    if trans is None or not np.any(trans):
        return np.array([minCrop] * 4, dtype=float)
    yend = -np.minimum(np.floor(trans[:, 0].min()), minCrop)
    xend = -np.minimum(np.floor(trans[:, 1].min()), minCrop)
    ystart = np.maximum(np.ceil(trans[:, 0].max()), minCrop)
    xstart = np.maximum(np.ceil(trans[:, 1].max()), minCrop)
    return np.array([ystart, xstart, yend, xend])


def tiled_frc(Image1, Image2, trans, box=(512, 512), overlap=0.5, dt=None):
    """Tiled Fourier ring correlation.  zorro.py:2246-2310."""
    if overlap > 0.8:
        overlap = 0.8
    crop = frc_crop_limits(trans)
    hann = apodization_hann(box).astype(dt.f)
    tilesX = int(np.floor(float(Image1.shape[1] - crop[1] - crop[3] - box[1]) / box[1] / (1.0 - overlap)))
    tilesY = int(np.floor(float(Image1.shape[0] - crop[0] - crop[2] - box[0]) / box[0] / (1.0 - overlap)))
    nc = np.float32(1.0 / (box[0] * box[1]) ** 2)
    FRC2D = np.zeros(box, dtype=dt.f)
    with np.errstate(all="ignore"):
        for I in range(max(tilesY, 0)):
            for J in range(max(tilesX, 0)):
                off = np.array([I * box[0] * (1.0 - overlap) + crop[0],
                                J * box[1] * (1.0 - overlap) + crop[1]]).astype(int)
                E = dt.fft2((hann * Image1[off[0]:off[0] + box[0], off[1]:off[1] + box[1]]).astype(dt.c)) * nc
                O = dt.fft2((hann * Image2[off[0]:off[0] + box[0], off[1]:off[1] + box[1]]).astype(dt.c)) * nc
                FRC2D += np.real(E * np.conj(O)) / np.sqrt(np.real(O * np.conj(O)) * np.real(E * np.conj(E)))
        FRC2D /= FRC2D[0, 0]
    FRC2D = np.fft.fftshift(FRC2D)
    return rotmean(FRC2D), FRC2D, (tilesY, tilesX)


def lazy_frc(images, translations, box=(512, 512), overlap=0.5, dt=None):
    """zorro.py:2226-2243."""
    even = np.sum(images[0::2], axis=0)
    odd = np.sum(images[1::2], axis=0)
    frc, frc2d, tiles = tiled_frc(even, odd, translations, box, overlap, dt)
    return frc[:int(box[0] / 2)], frc2d, tiles


def dose_filter_params(m, shapePadded, pixelsize, voltage, doseFiltParam, imageSum=None, dt=None):
    """Per-frame dose-filter constants.  zorro.py:2375-2452.  Returns the
    critical-dose constants, accumulated dose and per-frame thresQ."""
    f = dt.f
    A, B, Cc, order = (np.float32(doseFiltParam[i]) for i in (1, 2, 3, 4))
    vs = np.float32(np.sqrt(voltage / 300.0))
    N, Mx = shapePadded
    invPSx = np.float32(1.0 / (Mx * (pixelsize * 10)))
    invPSy = np.float32(1.0 / (N * (pixelsize * 10)))
    if doseFiltParam[0] is None:
        dosePerFrame = np.mean(imageSum) / m
    else:
        dosePerFrame = doseFiltParam[0]
    missingDose = dosePerFrame * np.float32(doseFiltParam[5])
    accum = np.zeros(m + 1, dtype=f)
    accum[1:] = np.cumsum(np.ones(m) * dosePerFrame)
    accum += missingDose
    qvect = (np.arange(0, shapePadded[0] / 2) * np.sqrt(invPSx * invPSy)).astype(f)
    opti = np.zeros(int(shapePadded[0] / 2), dtype=f)
    opti[1:] = np.float32(2.51284) * vs * (A * qvect[1:] ** B + Cc)
    opti[0] = opti[1] ** 2
    thresQ = np.empty(m)
    for J in range(m):
        idx = np.argwhere(np.abs(accum[J + 1] - opti) < np.abs(accum[J] - opti))
        thresQ[J] = qvect[idx[-1][0]]
    return {"A": A, "B": B, "C": Cc, "order": order, "vs": vs, "invPSx": invPSx, "invPSy": invPSy,
            "accum": accum, "thresQ": thresQ, "qvect": qvect}


def dose_filter_setup(m, shapePadded, pixelsize, voltage, doseFiltParam, imageSum, normalize=False, dt=None):
    """The frame-independent part of doseFilter (zorro.py:2375-2452): the
    constants, the q mesh and critical-dose map, the accumulators."""
    p = dose_filter_params(m, shapePadded, pixelsize, voltage, doseFiltParam, imageSum, dt)
    N, M = shapePadded
    xm, ym = np.meshgrid(np.arange(-M / 2, M / 2), np.arange(-N / 2, N / 2))
    xm = xm.astype(dt.f)
    ym = ym.astype(dt.f)
    with np.errstate(all="ignore"):
        qmesh = np.fft.fftshift(np.sqrt(xm * xm * (p["invPSx"] ** 2) + ym * ym * (p["invPSy"] ** 2)))
        crit = p["vs"] * (p["A"] * qmesh ** p["B"] + p["C"])
    crit[int(N / 2), int(M / 2)] = crit[int(N / 2), int(M / 2) - 1] ** 2
    return {"p": p, "qmesh": qmesh, "crit": crit, "shapePadded": shapePadded, "out_shape": imageSum.shape,
            "padW": np.array(shapePadded) - np.array(imageSum.shape), "acc": np.zeros(shapePadded, dtype=dt.c),
            "fmag": np.zeros(shapePadded, dtype=dt.f), "normalize": normalize, "dt": dt}


def dose_filter_add(st, frame, J):
    """Frame J's filtered spectrum added to the accumulator (the loop body of
    zorro.py:2455-2480)."""
    p, dt = st["p"], st["dt"]
    padW = st["padW"]
    with np.errstate(all="ignore"):
        filt = np.exp(np.float32(-0.5 * p["accum"][J + 1]) / st["crit"])
        thres = np.exp(-(st["qmesh"] / p["thresQ"][J]) ** p["order"])
        padded = np.pad(frame.astype(dt.c), ((0, padW[0]), (0, padW[1])), mode="symmetric")
        F = dt.fft2(padded)
        if st["normalize"]:
            cur = thres * filt
            st["fmag"] += cur
            st["acc"] += F * cur
        else:
            st["acc"] += F * thres * filt


def dose_filter_finish(st):
    """The inverse transform, abs and crop of doseFilter (zorro.py:2482-2494)."""
    dt = st["dt"]
    if st["normalize"]:
        out = dt.ifft2(st["acc"] * (np.float32(1.0) / (st["fmag"] + np.float32(1.0))))
    else:
        out = dt.ifft2(st["acc"])
    H, W = st["out_shape"]
    return np.abs(out[:H, :W])


def dose_filter(images, shapePadded, pixelsize, voltage, doseFiltParam, imageSum, normalize=False, dt=None):
    """Unblur-style dose-weighted sum.  zorro.py:2349-2494."""
    st = dose_filter_setup(images.shape[0], shapePadded, pixelsize, voltage, doseFiltParam, imageSum, normalize, dt)
    for J in range(images.shape[0]):
        dose_filter_add(st, images[J], J)
    return dose_filter_finish(st)


def psf_kernel(psf="K2", dt=None):
    """zorro.py:2511-2519."""
    p1 = 0.173235968 if psf == "K2" else 1.0
    psf = np.array([0.0, p1], dtype=dt.f)
    k = np.array([[psf[1] * psf[1], psf[1], psf[1] * psf[1]],
                  [psf[1], 0.0, psf[1]],
                  [psf[1] * psf[1], psf[1], psf[1] * psf[1]]], dtype=dt.f)
    return k / np.sum(k)


def hotpix_fit(unalignedSum, hotpixInfo, n_frames, dt):
    """Histogram, normal-CDF fit and sigma cut-offs.  zorro.py:2529-2602.

    Returns the fit and the updated hotpixInfo entries."""
    sumMean = np.mean(unalignedSum)
    poissonStd = np.sqrt(sumMean)
    histBins = np.arange(np.floor(sumMean - hotpixInfo["maxSigma"] * poissonStd) - 0.5,
                         np.ceil(sumMean + hotpixInfo["maxSigma"] * poissonStd) + 0.5, 1)
    hist, counts = np.histogram(unalignedSum, histBins)
    return hotpix_fit_from_hist(hist, counts, sumMean, poissonStd, hotpixInfo, dt)


def hotpix_fit_from_hist(hist, edges, sumMean, poissonStd, hotpixInfo, dt):
    """The host-side part of the hot-pixel statistics once the histogram is
    known.  zorro.py:2535-2592."""
    hist = hist.astype(dt.f)
    counts = edges[:-1].astype(dt.f)
    counts += 0.5 * (counts[1] - counts[0])
    cdf = np.cumsum(hist)
    cdf /= cdf[-1]

    def errorNormCDF(params):
        return np.sum(np.abs(cdf - scipy.stats.norm.cdf(counts, loc=params[0], scale=params[1])))

    best = scipy.optimize.minimize(errorNormCDF, (sumMean, poissonStd), method="L-BFGS-B",
                                   bounds=((sumMean - 0.5 * poissonStd, sumMean + 0.5 * poissonStd),
                                           (0.7 * poissonStd, 1.3 * poissonStd)))
    with np.errstate(all="ignore"):
        sigmaFromCDF = np.sqrt(2) * scipy.special.erfinv(2.0 * cdf - 1)
    normalSigma = (counts - best.x[0]) / best.x[1]
    err = normalSigma - sigmaFromCDF
    keep = ~np.isinf(err)
    err = err[keep]
    nsk = normalSigma[keep]
    info = {}
    # an empty fit raises, as np.linalg.lstsq did when the reference was
    # written, so the default cut-off is used (zorro.py:2572-2592)
    try:
        li = np.where(err > -0.5)[0][0]
        if li == 0:
            raise np.linalg.LinAlgError("empty lower fit")
        lf = np.linalg.lstsq(np.array([nsk[:li], np.ones(li)]).T, err[:li], rcond=None)[0]
        cutoffLower = np.float32(-lf[1] / lf[0])
        info["cutoffLower"] = float(cutoffLower)
    except Exception:
        cutoffLower = np.float32(hotpixInfo["cutoffLower"])
    try:
        ui = np.where(err < 0.5)[0][-1]
        if ui >= len(nsk):
            raise np.linalg.LinAlgError("empty upper fit")
        uf = np.linalg.lstsq(np.array([nsk[ui:], np.ones(len(nsk) - ui)]).T, err[ui:], rcond=None)[0]
        cutoffUpper = np.float32(-uf[1] / uf[0])
        info["cutoffUpper"] = float(cutoffUpper)
    except Exception:
        cutoffUpper = np.float32(hotpixInfo["cutoffUpper"])
    return {"mu": best.x[0], "sigma": best.x[1], "cutoffLower": cutoffLower, "cutoffUpper": cutoffUpper,
            "info": info}


def hotpix_filter(images, hotpixInfo, neighbourThres=0.01, dt=None):
    """Outlier-pixel filter.  zorro.py:2497-2672 (decorrOutliers off).

    Returns (filtered images, hotpixInfo updates, per-pixel maps)."""
    psfK = psf_kernel(hotpixInfo.get("psf", "K2"), dt)
    m = images.shape[0]
    unalignedSum = np.sum(images, axis=0)
    fit = hotpix_fit(unalignedSum, hotpixInfo, m, dt)
    info = dict(fit["info"])
    cL, cU = fit["cutoffLower"], fit["cutoffUpper"]
    sig = (unalignedSum - fit["mu"]) / fit["sigma"]
    info["guessDeadpix"] = int(np.sum(sig < cL))
    info["guessHotpix"] = int(np.sum(sig > cU))
    info["frameMean"] = float(fit["mu"] / m)
    info["frameStd"] = float(fit["sigma"] / np.sqrt(m))
    logK = np.float32(hotpixInfo["logisticK"])
    relax = np.float32(hotpixInfo["relax"])
    with np.errstate(all="ignore"):
        lm = 1.0 - 1.0 / (1.0 + np.exp(logK * (sig - cL * relax)))
        lm = (lm / (1.0 + np.exp(logK * (sig - cU * relax)))).astype(dt.f)
    conv = np.float32(1.0) - lm
    nom = (np.float32(1.0) - lm) * scipy.ndimage.convolve(np.float32(1.0) - lm, psfK)
    single = conv * (nom <= neighbourThres)
    mean_img = unalignedSum / m
    psfMean = scipy.ndimage.convolve(mean_img, psfK).astype(dt.f)
    nmask = nom > neighbourThres
    ys, xs = np.where(nmask)
    bestMean = fit["mu"] / m
    info["neighborPix"] = len(ys)
    nfilt = np.zeros_like(psfMean)
    with np.errstate(all="ignore"):
        for (y, x) in zip(ys, xs):
            hood = nmask[y - 1:y + 2, x - 1:x + 2]
            ratio = np.sum(hood) / hood.size
            if ratio > 0.66 or ratio <= 0.001 or np.isnan(ratio):
                nfilt[y, x] = bestMean
            else:
                nfilt[y, x] = conv[y, x] * np.mean(mean_img[y - 1:y + 2, x - 1:x + 2][~hood])
    out = lm * images + single * psfMean + nfilt
    return out, info, {"logisticMask": lm, "singleton": single, "psfFiltMean": psfMean,
                       "neighbourFilt": nfilt, "unalignedSum": unalignedSum, "sigma": sig, "fit": fit}


# --------------------------------------------------------------------------
# the whole call
# --------------------------------------------------------------------------

DEFAULTS = dict(shapeBinned=None, shapePadded=[4096, 4096], fouCrop=[3072, 3072], triMode="diag", diagWidth=5, diagStart=0,
                maxShift=100, preShift=False, autoMax=10, subPixReg=16, Bmode="opti", Brad=512, weightMode="autologistic",
                peaksigThres=6.0, logisticK=5.0, logisticNu=0.15, originMode="centroid",
                suppressOrigin=True, shiftMethod="lanczos", doLazyFRC=True, doEvenOddFRC=False, filterMode=None,
                doseFiltParam=[None, 0.24499, -1.6649, 2.8141, 32, 0], pixelsize=None, voltage=300.0,
                hotpixInfo={"logisticK": 6.0, "relax": 0.925, "maxSigma": 8.0, "psf": "K2",
                            "guessHotpix": 0, "guessDeadpix": 0, "decorrOutliers": False,
                            "cutoffLower": -4.0, "cutoffUpper": 3.25, "neighborPix": 0})


def half_set_sum(stack, o, translations, fp64=True, workers=1):
    """The aligned sum of a half set for given drift translations: the
    half-set registration's hot-pixel filter (when the settings have one) and
    applyShifts (zorro.py:1734-1808) without the correlation and the solve."""
    dt = Dtypes(fp64, workers)
    images = np.array(stack, copy=True)
    if "hot" in (o.get("filterMode") or "").lower():
        images, _, _ = hotpix_filter(images, dict(o["hotpixInfo"]), dt=dt)
    _, s = apply_shifts(images, translations, o["originMode"], o["shiftMethod"], o["subPixReg"],
                        shapePadded=o["shapePadded"], dt=dt)
    return s


def even_odd_frc(aligned, o, fp64=True, workers=1, half_trans=None, capture=None):
    """Independent half-set FRC.  zorro.py:2099-2224 (xcorr='tri').

    The even and odd frames of the aligned stack are registered again by two
    registrators with the parent's settings (its hot-pixel filter included;
    their own FRC and dose filter produce nothing that is kept, so they are
    not run), the two sums are aligned to each other with triMode 'first',
    and tiledFRC runs on that pair with the crop limits of
    hstack([transEven, transOdd]).  The sub-registrators do not recurse
    (doEvenOddFRC=False: the reference's own sub-registrators inherit
    doEvenOddFRC=True from the saved config and recurse until a half-set is
    too small for cdfLogisticCurve).  Returns FRC (full ring count), FRC2D,
    transEven, transOdd."""
    sub = dict(o)
    sub["doEvenOddFRC"] = False
    sub["doLazyFRC"] = False
    hot = "hot" in (o.get("filterMode") or "").lower()
    sub["filterMode"] = "hot" if hot else None
    if half_trans is None:
        ev = align_image_stack(aligned[0::2], fp64=fp64, workers=workers,
                               **dict(sub, hotpixInfo=dict(o["hotpixInfo"])))
        od = align_image_stack(aligned[1::2], fp64=fp64, workers=workers,
                               **dict(sub, hotpixInfo=dict(o["hotpixInfo"])))
        te, to = ev["translations"], od["translations"]
        se, so = ev["imageSum"], od["imageSum"]
        if capture is not None:
            capture["even"], capture["odd"] = ev["errorDict"], od["errorDict"]
    else:
        # the FRC that given half-set trajectories lead to (the half-set
        # registrations' correlation and solve replaced by ``half_trans``)
        te, to = (np.asarray(t) for t in half_trans)
        se = half_set_sum(aligned[0::2], sub, te, fp64, workers)
        so = half_set_sum(aligned[1::2], sub, to, fp64, workers)
    dt = Dtypes(fp64, workers)
    pair = np.stack([se, so]).astype(dt.f)
    eo = align_image_stack(pair, fp64=fp64, workers=workers,
                           **dict(sub, triMode="first", hotpixInfo=dict(o["hotpixInfo"])))
    trans = np.hstack([te, to])
    frc, frc2d, _ = tiled_frc(eo["images"][0], eo["images"][1], trans, dt=dt)
    return frc, frc2d, te, to


def align_image_stack(images, *, fp64=True, workers=1, capture=None, **attrs):
    """Restatement of ``alignImageStack`` for the 'zorro' xcorrMode with one
    (default) mask.  zorro.py:1569-1716.  ``images`` [N,H,W] (float32 as
    loadData delivers them) is copied, not modified.  Returns a dict of the
    outputs the reference leaves on the registrator."""
    o = dict(DEFAULTS)
    o["hotpixInfo"] = dict(DEFAULTS["hotpixInfo"])
    o.update(attrs)
    dt = Dtypes(fp64, workers)
    bench = {}
    images = np.array(images, copy=True)
    res = {}
    fm = (o["filterMode"] or "").lower()
    if o.get("shapeBinned") is not None and np.any(o["shapeBinned"]):
        # zorro.py:1588-1589 and 1834-1836: binned first, pixel size scaled
        scale = np.array(images.shape[1:]) / np.array(o["shapeBinned"])
        if o["pixelsize"] is not None:
            o["pixelsize"] = o["pixelsize"] * np.mean(scale)
        images = bin_stack(images, o["shapeBinned"], dt)
        res["pixelsize"] = o["pixelsize"]
    if "hot" in fm:
        bench["hot0"] = time.time()
        images, info, _ = hotpix_filter(images, o["hotpixInfo"], dt=dt)
        o["hotpixInfo"].update(info)
        res["hotpixInfo"] = o["hotpixInfo"]
        bench["hot1"] = time.time()
    N, H, W = images.shape
    P = o["shapePadded"]
    if o["shiftMethod"] == "fourier":
        # xcorrnm2_tri stores full spectra for this shift method and stops on
        # an undefined attribute while doing so (self.__sC2, zorro.py:891-895)
        raise AttributeError("shiftMethod 'fourier' is broken in the reference: self.__sC2 is undefined "
                             "(zorro.py:895)")
    padded, mask = pad_stack(images, P)
    bench["xcorr0"] = time.time()
    sh, co, ps, orig = xcorr_tri(padded, mask, shapePadded=P, fouCrop=o["fouCrop"], triMode=o["triMode"],
                                 diagWidth=o["diagWidth"], diagStart=o["diagStart"], maxShift=o["maxShift"],
                                 subPixReg=o["subPixReg"], Bmode=o["Bmode"], Brad=o["Brad"],
                                 suppressOrigin=o["suppressOrigin"], dt=dt, capture=capture,
                                 preShift=o.get("preShift", False), peaksigThres=o["peaksigThres"],
                                 autoMax=o.get("autoMax", 10))
    bench["xcorr3"] = time.time()
    if o["triMode"] == "first":
        translations = -sh[0, :]
        ed = {"shiftsTriMat": sh, "corrTriMat": co, "originTriMat": orig, "peaksigTriMat": ps,
              "translations": translations.copy()}
    elif o["triMode"] == "refine":
        # zorro.py:1635-1647: the diagonal, negated, in a float32 array
        translations = np.zeros([N, 2], dtype="float32")
        for K in range(N):
            translations[K, :] = -sh[K, K, :]
        ed = {"shiftsTriMat": sh, "corrTriMat": co, "originTriMat": orig, "peaksigTriMat": ps,
              "translations": translations.copy()}
    else:
        ed = shifts_solver(sh, co, ps, shapeImage=P, maxShift=o["maxShift"], weightMode=o["weightMode"],
                           peaksigThres=o["peaksigThres"], logisticK=o["logisticK"],
                           logisticNu=o["logisticNu"])
        ed["originTriMat"] = orig
        translations = ed["translations"].copy()
    bench["solve1"] = time.time()
    images = padded[:, :H, :W]
    t, imageSum = apply_shifts(images, translations, o["originMode"], o["shiftMethod"], o["subPixReg"],
                               shapePadded=P, dt=dt)
    bench["shifts1"] = time.time()
    res.update({"translations": t, "imageSum": imageSum, "errorDict": ed, "images": images})
    if o["doEvenOddFRC"]:
        halves = {}
        frc, frc2d, te, to = even_odd_frc(images, o, fp64=fp64, workers=workers, capture=halves)
        res.update({"FRC": frc, "FRC2D": frc2d, "transEven": te, "transOdd": to, "halfSetErrorDicts": halves,
                    "settings": o})
    elif o["doLazyFRC"]:
        frc, frc2d, tiles = lazy_frc(images, t, dt=dt)
        res.update({"FRC": frc, "FRC2D": frc2d, "frc_tiles": tiles})
    bench["frc1"] = time.time()
    for filt in fm.replace(" ", "").split(","):
        if filt in ("dose", "dosenorm"):
            res["filtSum"] = dose_filter(images, P, o["pixelsize"], o["voltage"], o["doseFiltParam"], imageSum,
                                         normalize=(filt == "dosenorm"), dt=dt)
    bench["dose1"] = time.time()
    res["bench"] = bench
    return res

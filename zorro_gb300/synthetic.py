"""Seeded synthetic cryo-EM movies with known drift.

There are no real detector movies here, so every test and benchmark input is
drawn from this generator.  It follows the recipe of the reference's drift
phantom (``zorro/scripts/analyticPhantom.py``) in spirit: a band-limited
random-phase specimen, a drift trajectory, Poisson counting noise.

* Specimen: white normal noise low-passed by ``exp(-f^2 / (2 sf^2))`` with
  ``sf = lowpass * 0.5`` cycles/px (``lowpass`` is the fraction of Nyquist),
  then ``1 + contrast * field / std(field)``.  It is drawn on a canvas larger
  than the detector by the largest drift so that no frame sees a wrap.
* Drift: a cumulative Gaussian random walk (``drift_sigma`` px per frame)
  plus i.i.d. ``N(0, jitter)`` jitter, centroid-zeroed.  Frame ``j`` is the
  specimen Fourier-shifted by ``drift[j]`` (exact sub-pixel), then cropped.
* Counts: ``Poisson(mean_dose * frame / gain)``.  With ``dtype='uint8'`` the
  counts are stored as bytes (clipped at 255), with ``'float16'`` as half
  floats (exact up to 2048); a multiplicative gain map ``U(0.9, 1.1)`` and a
  fraction of hot pixels at ``hot_factor * mean_dose`` counts are added when
  asked.

Every frame draws from its own random stream (spawned from ``seed``) and
transforms with the same FFT thread count, so frames are generated in
parallel threads (``workers``) with the same result for any thread count.

``images`` is what ``ImageRegistrator.alignImageStack`` receives after the
reference's ``loadData`` applies the gain: ``float32(gain * raw)``.
"""
from __future__ import annotations

import concurrent.futures
import os

import numpy as np
import scipy.fft


def _specimen(rng, shape, lowpass, contrast):
    noise = rng.standard_normal(shape, dtype=np.float32)
    F = scipy.fft.rfft2(noise, workers=-1)
    fy = np.fft.fftfreq(shape[0]).astype(np.float32)[:, None]
    fx = np.fft.rfftfreq(shape[1]).astype(np.float32)[None, :]
    sf = np.float32(lowpass * 0.5)
    F *= np.exp(-(fy * fy + fx * fx) / (2 * sf * sf))
    field = scipy.fft.irfft2(F, s=shape, workers=-1).astype(np.float32)
    field /= field.std()
    return (1.0 + contrast * field).astype(np.float32)


def drift_trajectory(rng, n_frames, drift_sigma, jitter=0.1):
    steps = rng.normal(0.0, drift_sigma, size=(n_frames, 2))
    steps[0] = 0.0
    walk = np.cumsum(steps, axis=0)
    walk += rng.normal(0.0, jitter, size=(n_frames, 2))
    walk -= walk.mean(axis=0)
    return walk


def make_movie(n_frames, shape, *, seed, mean_dose=1.0, drift_sigma=0.8, jitter=0.1,
               lowpass=1.0 / 8.0, contrast=0.1, dtype="float32", gain_map=False,
               hot_fraction=0.0, hot_factor=50.0, workers=None, with_images=True):
    """Return a dict with ``raw`` (counts), ``gain`` (or None), ``images``
    (float32 gain-corrected frames; None without ``with_images``), ``drift``
    ([N,2] y,x truth) and ``hot`` (flat indices of planted hot pixels)."""
    H, W = int(shape[0]), int(shape[1])
    rng = np.random.Generator(np.random.PCG64(seed))
    drift = drift_trajectory(rng, n_frames, drift_sigma, jitter)
    pad = int(np.ceil(np.abs(drift).max())) + 4
    cy = scipy.fft.next_fast_len(H + 2 * pad, real=True)
    cx = scipy.fft.next_fast_len(W + 2 * pad, real=True)
    spec = _specimen(rng, (cy, cx), lowpass, contrast)
    S = scipy.fft.rfft2(spec, workers=-1)
    fy = np.fft.fftfreq(cy).astype(np.float64)
    fx = np.fft.rfftfreq(cx).astype(np.float64)
    gain = rng.uniform(0.9, 1.1, size=(H, W)).astype(np.float32) if gain_map else None
    raw_dtype = {"uint8": np.uint8, "float16": np.float16}.get(dtype, np.float32)
    raw = np.empty((n_frames, H, W), dtype=raw_dtype)
    n_hot = int(round(hot_fraction * H * W))
    hot = np.sort(rng.choice(H * W, size=n_hot, replace=False)) if n_hot else np.zeros(0, dtype=np.int64)
    frame_rngs = [np.random.Generator(np.random.PCG64(s)) for s in
                  np.random.SeedSequence(seed).spawn(n_frames)]

    def one(j):
        dy, dx = drift[j]
        ramp = (np.exp(-2j * np.pi * fy * dy)[:, None] * np.exp(-2j * np.pi * fx * dx)[None, :]).astype(np.complex64)
        # every call with all cores: the split of rows between FFT threads
        # changes the last bits on some platforms, so it must not depend on
        # how many frames are in flight
        frame = scipy.fft.irfft2(S * ramp, s=(cy, cx), workers=-1)[pad:pad + H, pad:pad + W]
        lam = np.clip(mean_dose * frame, 0.0, None)
        if gain is not None:
            lam = lam / gain
        counts = frame_rngs[j].poisson(lam)
        if raw_dtype == np.uint8:
            counts = np.clip(counts, 0, 255)
        counts = counts.astype(raw_dtype)
        if n_hot:
            counts.reshape(-1)[hot] = raw_dtype(round(hot_factor * mean_dose))
        raw[j] = counts

    nw = max(1, min(n_frames, workers if workers is not None else (1 if H * W < (1 << 22) else (os.cpu_count() or 1))))
    if nw == 1:
        for j in range(n_frames):
            one(j)
    else:
        with concurrent.futures.ThreadPoolExecutor(nw) as ex:
            list(ex.map(one, range(n_frames)))
    if not with_images:
        images = None
    elif gain is not None:
        images = (gain[None, :, :] * raw.astype(np.float32)).astype(np.float32)
    else:
        images = raw.astype(np.float32)
    return {"raw": raw, "gain": gain, "images": images, "drift": drift, "hot": hot}

"""Named registration workloads: the synthetic movies and ImageRegistrator
settings that the benchmark and the parity tests run.

Each entry pairs the arguments of ``synthetic.make_movie`` (``movie``) with
the registrator attributes (``attrs``).  There is no public dataset for this
path, so every workload is a seeded synthetic movie with the shapes, counts
and drift of the configuration it stands for.

* ``config1`` -- 20 frames of 1024 x 1024 float32 counts (mean 1.0 e/px/frame),
  full triangle (190 pairs), padded and cropped at 1024, maxShift 40, dose
  filter at 1.0 e/A^2/frame and 1.0 A/px, Lanczos shift, independent even/odd
  FRC.
* ``k2`` -- 40 frames of 3838 x 3710 uint8 counts (mean 0.8) with a
  U(0.9, 1.1) gain map and 0.01 % hot pixels at 50x the mean, padded to 4096,
  Fourier-cropped to 2048 (780 pairs, maxShift 100), hot-pixel and dose
  filters (1.2 e/A^2/frame at 1.05 A/px), even/odd FRC.
* ``k2x10`` -- the K2 movie cut to 10 frames (142 MB of counts, still larger
  than L2).
* ``small`` -- ``config1`` without the even/odd FRC.
"""
from __future__ import annotations

K2_DOSE = [1.2 * 1.05 ** 2, 0.24499, -1.6649, 2.8141, 32, 0]
CONFIG1_DOSE = [1.0, 0.24499, -1.6649, 2.8141, 32, 0]

_K2_MOVIE = dict(n_frames=40, shape=(3838, 3710), seed=2024, mean_dose=0.8, drift_sigma=1.2, dtype="uint8",
                 gain_map=True, hot_fraction=1e-4, hot_factor=50.0)
_K2_ATTRS = dict(triMode="tri", shapePadded=[4096, 4096], fouCrop=[2048, 2048], maxShift=100, pixelsize=0.105,
                 voltage=300.0, filterMode="hot,dose", doseFiltParam=K2_DOSE, subPixReg=16, shiftMethod="lanczos",
                 Bmode="opti", doEvenOddFRC=True)
_C1_MOVIE = dict(n_frames=20, shape=(1024, 1024), seed=1, mean_dose=1.0, drift_sigma=0.8)
_C1_ATTRS = dict(triMode="tri", shapePadded=[1024, 1024], fouCrop=[1024, 1024], maxShift=40, pixelsize=0.1,
                 voltage=300.0, filterMode="dose", doseFiltParam=CONFIG1_DOSE, subPixReg=16, shiftMethod="lanczos",
                 Bmode="opti", doEvenOddFRC=True)

WORKLOADS = {
    "k2": dict(movie=dict(_K2_MOVIE), attrs=dict(_K2_ATTRS)),
    "k2x10": dict(movie=dict(_K2_MOVIE, n_frames=10), attrs=dict(_K2_ATTRS)),
    "config1": dict(movie=dict(_C1_MOVIE), attrs=dict(_C1_ATTRS)),
    "small": dict(movie=dict(_C1_MOVIE), attrs=dict(_C1_ATTRS, doEvenOddFRC=False)),
}


def workload(name):
    """(movie kwargs, attrs) of a named workload, as fresh copies."""
    wl = WORKLOADS[name]
    return dict(wl["movie"]), dict(wl["attrs"])

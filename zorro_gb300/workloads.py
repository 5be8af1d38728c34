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

``CONFIG4`` is the batched uneven workload: 16 movies of three detector
shapes in the proportions 8 / 5 / 3 -- K2 counting movies (40 x 3838 x 3710
uint8, mean 0.8, gain map and hot pixels), 4096 x 4096 float16 movies (30
frames, mean 1.5) and K3 super-resolution movies (50 x 8184 x 11520 uint8,
mean 0.25) Fourier-binned 2x to 4092 x 5760, each shape with its own drift
random-walk step drawn from U(0.5, 2.0) px/frame; full triangles, maxShift
100, dose filter, lazy FRC.
"""
from __future__ import annotations

import numpy as np

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


CONFIG4 = {
    "k2": dict(count=8, movie=dict(n_frames=40, shape=(3838, 3710), mean_dose=0.8, dtype="uint8", gain_map=True,
                                   hot_fraction=1e-4, hot_factor=50.0),
               attrs=dict(triMode="tri", shapePadded=[4096, 4096], fouCrop=[2048, 2048], maxShift=100,
                          pixelsize=0.105, voltage=300.0, filterMode="hot,dose", doseFiltParam=K2_DOSE, subPixReg=16)),
    "f16": dict(count=5, movie=dict(n_frames=30, shape=(4096, 4096), mean_dose=1.5, dtype="float16"),
                attrs=dict(triMode="tri", shapePadded=[4096, 4096], fouCrop=[2048, 2048], maxShift=100,
                           pixelsize=0.1, voltage=300.0, filterMode="dose", doseFiltParam=CONFIG1_DOSE, subPixReg=16)),
    "superres": dict(count=3, movie=dict(n_frames=50, shape=(8184, 11520), mean_dose=0.25, dtype="uint8"),
                     attrs=dict(triMode="tri", shapeBinned=[4092, 5760], shapePadded=[4096, 6144],
                                fouCrop=[2048, 3072], maxShift=100, pixelsize=0.0525, voltage=300.0,
                                filterMode="dose", doseFiltParam=CONFIG1_DOSE, subPixReg=16)),
}


def config4_movies(seed=404, with_images=False, n_frames=None):
    """One seeded movie of each CONFIG4 shape (drift step from U(0.5, 2.0))
    and the shapes' settings: {shape: (movie dict, attrs, count)}.  With
    ``n_frames`` every movie gets that many frames (a movie's first n frames
    are then a movie of n frames: the served workload draws its frame counts
    that way)."""
    from .synthetic import make_movie
    rng = np.random.default_rng(seed)
    out = {}
    for k, (name, spec) in enumerate(CONFIG4.items()):
        sigma = float(rng.uniform(0.5, 2.0))
        mk = dict(spec["movie"], seed=seed + k, drift_sigma=sigma)
        if n_frames is not None:
            mk["n_frames"] = int(n_frames)
        mv = make_movie(**mk, with_images=with_images)
        out[name] = (mv, dict(spec["attrs"]), spec["count"])
    return out


# The served workload: Poisson arrivals at each rate, shapes drawn 50/30/20
# from CONFIG4's three, frame counts uniform in [20, 60], 160 GB of device
# memory for the movies in flight.
CONFIG5 = {"rates": (0.5, 1.0, 2.0, 4.0), "mix": {"k2": 0.5, "f16": 0.3, "superres": 0.2},
           "frames": (20, 60), "hbm_budget": 160e9}

"""Continuous-batching movie registration on one GPU.

``MovieServer`` keeps several movies in flight at once.  Each admitted movie
runs ``ImageRegistrator.alignImageStack`` in a slot (a worker thread with its
own CUDA stream and device buffers); while one movie's host steps run (the
hot-pixel CDF fit, the drift solve) or its small kernels leave SMs idle,
the kernels of the others fill the GPU.  A request that arrives while all
slots are busy, or while the device memory it needs is not free under the
budget, waits in the queue and is admitted as soon as a slot and the memory
free up.  This replaces, on one GPU, what the reference's job daemon does
with one ``zorro -c`` process per movie (automator/zorroSkulkManager.py).

Every request's latency (submit to result) is recorded; ``stats()`` reports
movies/s and p50/p99 latency.  A request that fails (bad shape, a kernel
error) resolves its future with the exception; the other requests are not
affected.
"""
from __future__ import annotations

import collections
import concurrent.futures as cf
import copy
import threading
import time

import numpy as np

from .engine import Engine


def movie_bytes(reg, frames_shape, raw_itemsize):
    """Upper estimate of the device memory one movie needs (bytes)."""
    N, H, W = frames_shape
    P0, P1 = (int(reg.shapePadded[0]), int(reg.shapePadded[1])) if np.any(reg.shapePadded) else (H, W)
    C0, C1 = (int(2 * (v // 2)) for v in reg.fouCrop) if np.any(reg.fouCrop) else (P0, P1)
    K4 = ((C1 // 2 + 1) + 3) & ~3
    se = K4 * (C0 + 4)
    w = 2 * int(reg.maxShift)
    M = N * (N - 1) // 2
    filt = (reg.filterMode or "").lower()
    b = N * H * W * raw_itemsize                 # frames
    b += 2 * N * se * 8 + se * 8                 # spectra
    b += (4 * N + 1 + M) * w * w * 4             # windows
    b += 8 * H * W * 4                           # sums, maps
    from .engine import DOSE_WORK, SPECTRA_WORK, XCORR_WORK
    b += SPECTRA_WORK + XCORR_WORK
    if "dose" in filt or reg.keepAlignedImages:
        b += N * H * W * 4                       # aligned frames
    if "dose" in filt:
        b += DOSE_WORK
    b += 256 << 20                               # FRC, peaks, small buffers
    if getattr(reg, "doEvenOddFRC", False) and N >= 4:
        # the even and odd halves are registered again at the same time, each
        # on its own slot, from float32 aligned frames
        half = copy.copy(reg)
        half.doEvenOddFRC = False
        half.keepAlignedImages = False
        half.filterMode = "hot" if "hot" in filt else None
        b += 2 * movie_bytes(half, (N // 2, H, W), 4)
    return int(b)


class MovieServer:
    """Register movies concurrently on one GPU.

    ``slots``: movies in flight at most; ``hbm_budget``: device bytes the
    in-flight movies may hold together (admission control)."""

    def __init__(self, device=0, slots=2, hbm_budget=160e9):
        self.engine = Engine.get(device)
        self.device = device
        self.slots = int(slots)
        self.budget = float(hbm_budget)
        self._free_slots = collections.deque(range(1, self.slots + 1))
        self._in_use = 0.0
        self._cv = threading.Condition()
        self._pool = cf.ThreadPoolExecutor(max_workers=self.slots, thread_name_prefix="zorro-slot")
        self._lat = []
        self._done = 0
        self._t0 = None
        self._t1 = None
        self._closed = False

    def _acquire(self, need):
        with self._cv:
            while not self._free_slots or (self._in_use > 0 and self._in_use + need > self.budget):
                if self._closed:
                    raise RuntimeError("server closed")
                self._cv.wait()
            if need > self.budget:
                raise MemoryError("movie needs %.1f GB, more than the %.1f GB budget" % (need / 1e9, self.budget / 1e9))
            self._in_use += need
            return self._free_slots.popleft()

    def _release(self, slot, need):
        with self._cv:
            self._in_use -= need
            self._free_slots.append(slot)
            self._cv.notify_all()

    def _run(self, reg, t_submit):
        from .mrc import Packed4
        imgs = reg.images
        shape = tuple(imgs.shape)
        if isinstance(imgs, Packed4):
            itemsize = 1.5  # the packed bytes and the uint8 frames they expand into
        elif hasattr(imgs, "element_size"):
            itemsize = imgs.element_size()
        else:
            itemsize = np.asarray(imgs).dtype.itemsize
        need = movie_bytes(reg, shape, itemsize)
        slot = self._acquire(need)
        try:
            self.engine.align(reg, slot=slot)
        finally:
            self._release(slot, need)
        t = time.perf_counter()
        with self._cv:
            self._lat.append(t - t_submit)
            self._done += 1
            self._t1 = t
        return reg

    def submit(self, reg):
        """Queue one registrator; returns a Future resolving to it."""
        t = time.perf_counter()
        with self._cv:
            if self._t0 is None:
                self._t0 = t
        return self._pool.submit(self._run, reg, t)

    def stats(self):
        with self._cv:
            lat = np.array(self._lat)
            span = (self._t1 - self._t0) if (self._t0 is not None and self._t1 is not None) else float("nan")
            n = self._done
        return {"movies": n, "movies_per_s": n / span if span and span > 0 else float("nan"),
                "p50_s": float(np.percentile(lat, 50)) if n else float("nan"),
                "p99_s": float(np.percentile(lat, 99)) if n else float("nan")}

    def reset_stats(self):
        with self._cv:
            self._lat = []
            self._done = 0
            self._t0 = self._t1 = None

    def close(self):
        with self._cv:
            self._closed = True
            self._cv.notify_all()
        self._pool.shutdown(wait=True)

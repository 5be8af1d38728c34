"""The GPU pipeline behind ``ImageRegistrator.alignImageStack``.

One ``Engine`` per device owns the stream and a pool of device buffers
(PyTorch tensors, grown on demand and reused across movies); every pass over
pixels is a ``libzorrogb`` entry point.  Host work is limited to the float64
fits of ``hostmath`` and happens at three points where the reference's own
logic needs scalars: the hot-pixel histogram fit, the drift solve, and the
per-frame dose constants.

Two exact reformulations of the reference's arithmetic are used:

* each frame's mean (over the image area) is subtracted before the forward
  transforms when the mask is the default padStack mask.  The masked
  normalised correlation of zorro.py:1034-1074 is invariant to adding a
  constant inside a binary mask (the numerator minus CorrTM*CorrBM/maskProduct
  and both Denominator terms are covariances), so this changes only rounding:
  it removes the large mean-times-mean term that float32 would otherwise
  cancel;
* the four frame-only IFFTs of mnxc2 are computed once per frame, not once
  per pair.
"""
from __future__ import annotations

import concurrent.futures
import contextlib
import ctypes as C
import threading
import time
import types

import numpy as np

from . import _lib
from . import hostmath as hm
from ._lib import Frames, HotpixParams, PeakParams, PeakResult, DoseParams

# host view of zr_peak_result_t
_PEAK_DTYPE = np.dtype([("sy", "f8"), ("sx", "f8"), ("sigma", "f8"), ("corr", "f4"), ("peaksig", "f4"),
                        ("origin", "f4"), ("cy", "i4"), ("cx", "i4"), ("flags", "i4"), ("nfev", "i4")], align=True)

_RAW_TYPES = {np.dtype(np.float32): _lib.ZR_F32, np.dtype(np.uint8): _lib.ZR_U8, np.dtype(np.uint16): _lib.ZR_U16,
              np.dtype(np.float16): _lib.ZR_F16}

# scratch budgets (bytes) for the staged passes.  The pair stage runs its
# jobs in waves that fit XCORR_WORK, and every wave reads the spectra of all
# frames again: 1.5 GB holds the 780 pairs of a 40-frame K2 movie (1.6 MB of
# column-pass output each at crop 2048, maxShift 100) in one wave.
SPECTRA_WORK = 512 << 20
XCORR_WORK = 1536 << 20
DOSE_WORK = 1536 << 20


def _crop_ok(v):
    return (_pow2(v) and 64 <= v <= 4096) or v in (384, 768, 1536, 3072)


def _padded_ok(v):
    return (_pow2(v) and 64 <= v <= 4096) or v in (1536, 3072, 6144)


_CROP_OK, _PADDED_OK = _crop_ok, _padded_ok


def _pow2(v):
    return v > 0 and (v & (v - 1)) == 0


class Engine:
    _engines = {}

    @classmethod
    def get(cls, device=0):
        e = cls._engines.get(device)
        if e is None:
            e = cls._engines[device] = Engine(device)
        return e

    def __init__(self, device=0):
        import torch
        if not torch.cuda.is_available():
            raise _lib.ZorroError("no CUDA device: the GB300 registration path has no CPU fallback")
        self.torch = torch
        self.device = device
        self.dev = torch.device("cuda", device)
        self.lib = _lib.load()
        with torch.cuda.device(self.dev):
            _lib.call("zr_init", device)
        self._slots = {}
        self._slots_lock = threading.Lock()
        self._planned = set()
        self._plan_lock = threading.Lock()
        self.last_plan = None
        self._tls = threading.local()
        self.profile = None  # dict stage -> list of (start, end) CUDA events when enabled
        self._profile_lock = threading.Lock()

    def call(self, stage, name, *args):
        """One C-ABI call; bracketed by CUDA events on the current stream when
        profiling is on (self.profile is a dict)."""
        if self.profile is None:
            return _lib.call(name, *args)
        torch = self.torch
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        rc = _lib.call(name, *args)
        e1.record()
        with self._profile_lock:
            self.profile.setdefault(stage, []).append((e0, e1))
        return rc

    def stage_ms(self):
        """Summed device time per stage of the recorded calls (synchronises)."""
        self.torch.cuda.synchronize(self.dev)
        return {k: sum(a.elapsed_time(b) for a, b in v) for k, v in (self.profile or {}).items()
                if not k.startswith("host:")}

    def host_ms(self):
        """Summed host time of the host steps (CDF fits, drift solves) while
        profiling was on."""
        return {k[5:]: 1e3 * sum(b - a for a, b in v) for k, v in (self.profile or {}).items()
                if k.startswith("host:")}

    def host_intervals(self):
        """(step, start, end) of every host step while profiling was on, in
        time.perf_counter seconds."""
        return sorted((k[5:], a, b) for k, v in (self.profile or {}).items() if k.startswith("host:") for a, b in v)

    def _host_time(self, step, t0):
        if self.profile is not None:
            with self._profile_lock:
                self.profile.setdefault("host:" + step, []).append((t0, time.perf_counter()))

    # ------------------------------------------------------------------ planning
    def plan(self, P0, P1, C0, C1, mS, effort="FFTW_MEASURE", cache_dir=None):
        """Launch variants of the transform kernels for one registration shape
        (pyFFTWPlanner's FFTW_MEASURE planning and wisdom,
        zorro_util.py:966-1066): the choice saved in ``cache_dir``'s plan file
        for this GPU model and library version, or measured now by zr_plan
        and saved there.  'FFTW_ESTIMATE' keeps the built-in variants.  Done
        once per shape and engine; the variants change no result."""
        import json
        import os
        import tempfile
        if str(effort).upper() == "FFTW_ESTIMATE":
            return None
        key = (P0, P1, C0, C1, mS)
        with self._plan_lock:
            if key in self._planned:
                return None
            torch = self.torch
            shape = _lib.PlanShape(P0, P1, C0, C1, mS, 8)
            choice = _lib.PlanChoice()
            path = os.path.join(cache_dir or tempfile.gettempdir(), "zorro_gb300_plans.json")
            name = "%s|lib%d|P%dx%d|C%dx%d|m%d" % (torch.cuda.get_device_name(self.device), self.lib.zr_version(),
                                                   P0, P1, C0, C1, mS)
            try:
                with open(path) as fh:
                    wisdom = json.load(fh)
            except (OSError, ValueError):
                wisdom = {}
            saved = wisdom.get(name)
            if saved:
                choice.fwd_rows, choice.fwd_cols, choice.xc_cols, choice.xc_rows = (int(v) for v in saved["choice"])
                _lib.call("zr_plan_set", C.byref(shape), C.byref(choice))
            else:
                wb = self.lib.zr_plan_work_bytes(C.byref(shape))
                work = torch.empty(max(int(wb), 1), dtype=torch.uint8, device=self.dev)
                with torch.cuda.device(self.dev):
                    _lib.call("zr_plan", C.byref(shape), work.data_ptr(), wb,
                              torch.cuda.current_stream(self.dev).cuda_stream, C.byref(choice))
                del work
                wisdom[name] = {"choice": [choice.fwd_rows, choice.fwd_cols, choice.xc_cols, choice.xc_rows],
                                "ms_spectra": [list(r) for r in choice.ms_spectra],
                                "ms_pairs": [list(r) for r in choice.ms_pairs]}
                try:
                    tmp = "%s.%d.tmp" % (path, os.getpid())
                    with open(tmp, "w") as fh:
                        json.dump(wisdom, fh, indent=1, sort_keys=True)
                    os.replace(tmp, path)
                except OSError:
                    pass  # an unwritable cache directory only costs the next process a measurement
            self._planned.add(key)
            self.last_plan = (name, [choice.fwd_rows, choice.fwd_cols, choice.xc_cols, choice.xc_rows])
            return self.last_plan

    # ------------------------------------------------------------------ slots and buffers
    def _slot(self, slot, priority=0):
        """Per-slot state: a buffer pool and (except slot 0, which uses the
        caller's current stream) a stream of its own, made with ``priority``
        (negative: ahead of the other streams' kernels) on first use.  Movies
        registered in different slots can run concurrently from different
        threads."""
        with self._slots_lock:
            st = self._slots.get(slot)
            if st is None:
                stream = None if slot == 0 else self.torch.cuda.Stream(device=self.dev, priority=priority)
                st = self._slots[slot] = {"bufs": {}, "stream": stream, "key": slot}
            return st

    def _copy_stream(self):
        """A stream of the current slot for copies that may overlap its
        kernels (made on first use)."""
        st = getattr(self._tls, "slot", None) or self._slot(0)
        with self._slots_lock:
            s = st.get("copy")
            if s is None:
                s = st["copy"] = self.torch.cuda.Stream(device=self.dev)
            return s

    @property
    def bufs(self):
        st = getattr(self._tls, "slot", None)
        return st["bufs"] if st is not None else self._slot(0)["bufs"]

    def slot_bytes(self, slot=None):
        """Device bytes held by one slot's buffers (all slots when None)."""
        with self._slots_lock:
            slots = list(self._slots.values()) if slot is None else [self._slots.get(slot, {"bufs": {}})]
        return sum(t.numel() for st in slots for t in st["bufs"].values())

    def buf(self, name, nbytes):
        bufs = self.bufs
        t = bufs.get(name)
        if t is None or t.numel() < nbytes:
            if t is not None:
                del bufs[name]
                t = None
            t = self.torch.empty(max(int(nbytes), 1), dtype=self.torch.uint8, device=self.dev)
            bufs[name] = t
        return t

    def ptr(self, name, nbytes):
        return self.buf(name, nbytes).data_ptr()

    def tensor(self, name, shape, dtype):
        torch = self.torch
        n = int(np.prod(shape)) * torch.empty(0, dtype=dtype).element_size()
        return self.buf(name, n)[:n].view(dtype).view(*shape)

    @property
    def stream(self):
        return self.torch.cuda.current_stream(self.dev).cuda_stream

    # ------------------------------------------------------------------ input
    def upload(self, reg, pfx=""):
        torch = self.torch
        imgs = reg.images
        from .mrc import Packed4
        if isinstance(imgs, Packed4):
            # 4-bit movie: the packed bytes cross the host link, the device
            # expands them into the uint8 frames the kernels read
            N, H, W = imgs.shape
            src = torch.from_numpy(np.ascontiguousarray(imgs.data).reshape(-1))
            packed = self.buf(pfx + "u4packed", src.numel())[:src.numel()]
            packed.copy_(src, non_blocking=True)
            imgs = self.tensor(pfx + "u4frames", (N, H, W), torch.uint8)
            self.call("A_gain_sum", "zr_unpack_u4", packed.data_ptr(), N, H, W, imgs.data_ptr(), self.stream)
        if isinstance(imgs, torch.Tensor):
            t = imgs.to(self.dev, non_blocking=True)
            dt = np.dtype(str(t.dtype).replace("torch.", ""))
        else:
            a = np.ascontiguousarray(imgs)
            if a.dtype == np.float64:
                a = a.astype(np.float32)
            dt = a.dtype
            t = torch.from_numpy(a).to(self.dev, non_blocking=True)
        if t.ndim != 3:
            raise ValueError("zorro.alignImageStack: stacks must be 3D data")
        if dt not in _RAW_TYPES:
            raise ValueError("images dtype %s not supported (float32, uint8, uint16, float16)" % dt)
        # a selection of frames with contiguous rows (the even or odd frames of
        # an aligned stack) is read in place through the frame stride, when
        # its start and stride keep the kernels' 16-byte vector loads aligned
        N_, H_, W_ = (int(v) for v in t.shape)
        in_place = (t.is_cuda and t.stride(2) == 1 and t.stride(1) == W_ and t.stride(0) >= H_ * W_
                    and t.stride(0) % 4 == 0 and t.data_ptr() % 16 == 0)
        if not in_place:
            t = t.contiguous()
        gain = None
        raw_float = bool(getattr(reg, "imagesAreRaw", False))  # float frames read by loadData, gain not applied
        if reg.gainRef is not None and (dt != np.dtype(np.float32) or raw_float):
            g = reg.gainRef
            gain = (g.to(self.dev) if isinstance(g, torch.Tensor) else torch.from_numpy(
                np.ascontiguousarray(g, dtype=np.float32)).to(self.dev, non_blocking=True)).float().contiguous()
            if tuple(gain.shape) != tuple(t.shape[1:]):
                raise ValueError("gainRef shape %s does not match frames %s" % (tuple(gain.shape), tuple(t.shape[1:])))
        return t, gain, _RAW_TYPES[dt]

    # ------------------------------------------------------------------ pipeline
    def align(self, reg, slot=0):
        """Register one movie (all outputs set on ``reg``).  ``slot`` selects
        the buffer pool and stream; one thread per slot at a time."""
        torch = self.torch
        st = self._slot(slot)
        prev = getattr(self._tls, "slot", None)  # a half-set registration runs inside its parent's
        self._tls.slot = st
        try:
            sctx = torch.cuda.stream(st["stream"]) if st["stream"] is not None else contextlib.nullcontext()
            with torch.cuda.device(self.dev), sctx:
                res = self._align(reg)
                if st["stream"] is not None:
                    st["stream"].synchronize()
        finally:
            self._tls.slot = prev
        for k, v in res.items():
            setattr(reg, k, v)

    def _even_odd_frc(self, reg, aligned, hotinfo, filt, ready=None):
        """Independent half-set FRC (evenOddFouRingCorr, zorro.py:2099-2224,
        xcorr='tri').  The even and odd frames of the aligned stack are
        registered again with the parent's settings (its hot-pixel filter
        included; their own FRC and dose filter would produce nothing that is
        kept, so they are not run), their sums are aligned to each other in
        triMode 'first', and the tiled FRC of that pair uses the crop limits
        of hstack([transEven, transOdd]).  The half-set registrators do not
        recurse (the reference's own inherit doEvenOddFRC=True from the saved
        config and recurse until a half-set is too small to fit).  Returns
        FRC (all rings), FRC2D, transEven, transOdd and the half-set
        registrations' error dictionaries ({'even': ..., 'odd': ...}; the
        reference discards its half-set registrators, this keeps their pair
        measurements for inspection)."""
        torch = self.torch
        N, H, W = (int(v) for v in aligned.shape)
        if N < 2:
            raise ValueError("doEvenOddFRC needs at least two frames")
        # the half-set registrations read the aligned stack on their own streams,
        # after ``ready`` (recorded once the stack was written)
        if ready is None:
            ready = torch.cuda.Event()
            ready.record()
        parent = self._tls.slot["key"]

        def register(images, sub_slot, after_hot=None, start=None, **kw):
            r = self._half_set_reg(reg, images, hotinfo, filt, **kw)
            if start is not None:
                start.wait()
            # the half sets are on the critical path, the parent's dose filter
            # is not: their streams go first and the dose fills the gaps
            self._slot(sub_slot, priority=-1)["stream"].wait_event(ready)
            self._tls.after_hot = after_hot
            try:
                self.align(r, slot=sub_slot)
            finally:
                self._tls.after_hot = None
            return r

        # the two halves are independent: the odd one on a second slot (its own
        # stream and buffers) in a helper thread, started once the even one has
        # passed its hot-pixel fit, so that each half's host steps (hot-pixel
        # fit, drift solve) overlap the other's kernels instead of each other
        go = threading.Event()
        with concurrent.futures.ThreadPoolExecutor(1) as ex:
            fut = ex.submit(register, aligned[1::2], ("halfset_odd", parent), start=go)
            try:
                ev = register(aligned[0::2], ("halfset_even", parent), after_hot=go.set)
            finally:
                go.set()  # also when the even half failed before its hot-pixel step
            od = fut.result()
        # the half sums are complete (each half-set stream was synchronised):
        # stack them on the stream that registers the pair, not on the parent's,
        # whose low-priority dose kernels may still be queued ahead of the copy
        with torch.cuda.stream(self._slot(("halfset_even", parent), priority=-1)["stream"]):
            pair = torch.stack([ev.imageSum, od.imageSum])
        eo = register(pair, ("halfset_even", parent), triMode="first", keepAlignedImages=True)
        return self._pair_frc(ev, od, eo, H, W)

    @staticmethod
    def _half_set_reg(reg, images, hotinfo, filt, **kw):
        """A registrator for one half set of the even/odd FRC (or for the pair
        of half sums): the parent's settings, its fitted hot-pixel settings,
        no FRC and no dose filter of its own, outputs left on the device."""
        from .registrator import ImageRegistrator, copy_config
        r = ImageRegistrator()
        copy_config(reg, r)
        r.images = images
        r.gainRef = None
        r.masks = None
        r.gain = None
        r.doEvenOddFRC = False
        r.doLazyFRC = False
        r.filterMode = "hot" if "hot" in filt else None
        r.hotpixInfo = dict(hotinfo)
        r.keepAlignedImages = False
        r.returnDeviceArrays = True
        r.errorDictList = []
        r.bench = {}
        for k, v in kw.items():
            setattr(r, k, v)
        return r

    def _pair_frc(self, ev, od, eo, H, W, pfx=""):
        """The tiled FRC of the aligned pair of half sums (``eo``, registered in
        triMode 'first') with the crop limits of hstack([transEven,
        transOdd]).  Returns FRC, FRC2D, transEven, transOdd and the half-set
        error dictionaries."""
        torch = self.torch
        te, to = np.asarray(ev.translations), np.asarray(od.translations)
        box = 512
        offs, tiles = hm.frc_tiles((H, W), np.hstack([te, to]))
        nr = int(np.ceil(np.sqrt(2.0 * (box // 2) ** 2))) + 1
        if len(offs) and (offs.min() < 0 or (offs[:, 0] + box).max() > H or (offs[:, 1] + box).max() > W):
            raise ValueError("tiledFRC: tiles %s leave the %dx%d image (negative crop limits)" % (tiles, H, W))
        halves = {"even": ev.errorDictList[-1], "odd": od.errorDictList[-1]}
        if len(offs) == 0:
            return np.full(nr, np.nan), np.full((box, box), np.nan, dtype=np.float32), te, to, halves
        pair = eo.images.contiguous()
        offs_dev = torch.from_numpy(offs.reshape(-1)).to(self.dev, non_blocking=True)
        fwb = self.lib.zr_frc_work_bytes(len(offs), box)
        f2 = self.tensor(pfx + "frc2d", (box, box), torch.float32)
        fr = self.tensor(pfx + "frc_eo", (nr,), torch.float64)
        self.call("H_frc", "zr_tiled_frc", pair[0].data_ptr(), pair[1].data_ptr(), H, W, box, offs_dev.data_ptr(),
                  len(offs), f2.data_ptr(), fr.data_ptr(), nr, self.ptr(pfx + "frcwork", fwb), fwb, self.stream)
        return fr, f2, te, to, halves

    # ------------------------------------------------------------------ batches of movies
    def align_batch(self, regs, slot=0):
        """Register several movies, of any detector sizes and frame counts,
        with shared launches (all outputs set on each registrator).

        Each movie is prepared on its own (upload, Fourier binning, hot-pixel
        filter); movies of the same shape class (frame shape, pixel type,
        corrections, transform sizes, peak search: ``batch_key``) then share
        one set of launches for the forward spectra, the frame terms, the
        correlation windows of every pair and their peak search, their frames
        concatenated and each frame reading its own movie's maps.  Each movie
        is then solved, shifted and filtered; the half sets of every movie's
        even/odd FRC are registered as one more batch, and the pairs of their
        sums as another.  The results equal each movie registered alone
        (the same kernels on the same values; tested)."""
        torch = self.torch
        st = self._slot(slot)
        prev = getattr(self._tls, "slot", None)
        self._tls.slot = st
        try:
            sctx = torch.cuda.stream(st["stream"]) if st["stream"] is not None else contextlib.nullcontext()
            with torch.cuda.device(self.dev), sctx:
                outs = self._align_batch(regs, "b")
                if st["stream"] is not None:
                    st["stream"].synchronize()
        finally:
            self._tls.slot = prev
        for reg, res in zip(regs, outs):
            for k, v in res.items():
                setattr(reg, k, v)

    def _align_batch(self, regs, tag):
        jobs = [self._prepare(r, pfx="%s%d_" % (tag, i)) for i, r in enumerate(regs)]
        classes = {}
        for j in jobs:
            key = self.batch_key(j)
            classes.setdefault(key if key is not None else ("alone", j.pfx), []).append(j)
        for ci, js in enumerate(classes.values()):
            self._correlate(js, cls="%sc%d_" % (tag, ci))
        outs = [self._finish_main(j) for j in jobs]
        eo = [j for j in jobs if j.reg.doEvenOddFRC]
        halves = dict(zip((j.pfx for j in eo), self._even_odd_batch(eo, tag))) if eo else {}
        return [self._finish_out(j, out, halves.get(j.pfx)) for j, out in zip(jobs, outs)]

    def _even_odd_batch(self, jobs, tag):
        """The independent even/odd FRC of several movies: every movie's even
        and odd half sets registered as one batch, the pairs of half sums as
        another, then each movie's tiled FRC (as _even_odd_frc does for one)."""
        torch = self.torch
        halves = []
        for j in jobs:
            if j.N < 2:
                raise ValueError("doEvenOddFRC needs at least two frames")
            halves.append(self._half_set_reg(j.reg, j.aligned[0::2], j.hotinfo, j.filt))
            halves.append(self._half_set_reg(j.reg, j.aligned[1::2], j.hotinfo, j.filt))
        self._set_outputs(halves, self._align_batch(halves, tag + "h"))
        pairs = []
        for k, j in enumerate(jobs):
            pair = torch.stack([halves[2 * k].imageSum, halves[2 * k + 1].imageSum])
            pairs.append(self._half_set_reg(j.reg, pair, j.hotinfo, j.filt, triMode="first", keepAlignedImages=True))
        self._set_outputs(pairs, self._align_batch(pairs, tag + "f"))
        return [self._pair_frc(halves[2 * k], halves[2 * k + 1], pairs[k], j.H, j.W, pfx=j.pfx)
                for k, j in enumerate(jobs)]

    @staticmethod
    def _set_outputs(regs, outs):
        for reg, res in zip(regs, outs):
            for k, v in res.items():
                setattr(reg, k, v)

    def _frames(self, raw, rtype, gain, ha=None, hb=None, gdiv=0.0):
        N, H, W = raw.shape
        return Frames(raw.data_ptr(), rtype, gain.data_ptr() if gain is not None else None,
                      ha.data_ptr() if ha is not None else None, hb.data_ptr() if hb is not None else None,
                      float(gdiv), N, H, W, int(raw.stride(0)))

    def _cropped_peaks(self, reg, pairs, refine, N, C0, C1, mS, pp, spec, st):
        """The +/-maxShift correlation windows of every pair (mnxc2,
        zorro.py:1014-1097) and their peaks (locatePeak, one CTA a window).
        Returns the peak records, one per pair."""
        torch = self.torch
        half, G, S, GM, G16, S16, GM16, hsc = spec
        M = len(pairs)
        w = 2 * mS
        se = int(GM.shape[0])
        terms = self.tensor("terms", (4 * N + 1, w, w), torch.float32)
        xw = min(XCORR_WORK, max(self.lib.zr_xcorr_work_bytes(1, C1, mS), self.lib.zr_xcorr_work_bytes(M, C1, mS)))
        xptr = self.ptr("xcwork", xw)
        if half:
            # products, inverse transforms and the combination stay float32
            self.call("D_frame_terms", "zr_xcorr_terms_half", G16.data_ptr(), S16.data_ptr(), GM16.data_ptr(),
                      hsc.data_ptr(), N, C0, C1, mS, terms.data_ptr(), xptr, xw, st)
        else:
            self.call("D_frame_terms", "zr_xcorr_terms", G.data_ptr(), S.data_ptr(), GM.data_ptr(), N, C0, C1, mS,
                      terms.data_ptr(), xptr, xw, st)
        cwin = self.tensor("cwin", (max(M, 1), w, w), torch.float32)
        if refine:
            TG = self.tensor("refineT", (N, se, 2), torch.float32)
            rterms = self.tensor("refine_terms", (4 * N + 1, w, w), torch.float32)
            self.call("E_pairs", "zr_refine_spectra", G.data_ptr(), N, C0, C1, TG.data_ptr(), st)
            self.call("E_pairs", "zr_refine_terms", terms.data_ptr(), N, mS, rterms.data_ptr(), st)
            self.call("E_pairs", "zr_xcorr_refine", G.data_ptr(), TG.data_ptr(), rterms.data_ptr(), N, C0, C1, mS,
                      cwin.data_ptr(), xptr, xw, st)
        elif half:
            pairs_dev = torch.from_numpy(pairs.reshape(-1)).to(self.dev, non_blocking=True)
            self.call("E_pairs", "zr_xcorr_pairs_half", G16.data_ptr(), hsc.data_ptr(), terms.data_ptr(),
                      pairs_dev.data_ptr(), M, N, C0, C1, mS, cwin.data_ptr(), xptr, xw, st)
        else:
            pairs_dev = torch.from_numpy(pairs.reshape(-1)).to(self.dev, non_blocking=True)
            self.call("E_pairs", "zr_xcorr_pairs", G.data_ptr(), terms.data_ptr(), pairs_dev.data_ptr(), M, N, C0, C1,
                      mS, cwin.data_ptr(), xptr, xw, st)
        pres = self.tensor("peaks", (max(M, 1), C.sizeof(PeakResult)), torch.uint8)
        self.call("F_peaks", "zr_locate_peaks", cwin.data_ptr(), M, mS, C.byref(pp), pres.data_ptr(), st)
        host = pres[:M].cpu().numpy()
        return np.frombuffer(host.tobytes(), dtype=_PEAK_DTYPE).copy()

    def _preshift(self, reg, pairs, refine, N, C0, C1, pp, spec, st):
        """preShift (zorro.py:1089-1092, 1148-1168): whole C x C correlation
        planes, searched within the maxShift disc rolled to the rounded shift
        of the previous pair of the row (shiftsTriMat[I, J-1], in cropped
        pixels as measured so far; 'refine': shiftsTriMat[I-1, I-1]).  A pair
        depends only on its left neighbour in its row, so the pairs go
        diagonal by diagonal (all J - I = d together; 'refine' one frame at a
        time).  The planes of a diagonal are searched together: the host
        steps the bounded Brent search over sigma of every plane in lock
        step, each step one batched filter launch.  Returns the peak records
        and which pairs were measured ('auto' stops a row as the reference
        does)."""
        import math
        torch = self.torch
        if C0 != C1:
            raise ValueError("preShift needs a square Fourier crop: the reference builds its search mask with the "
                             "crop's axes swapped (zorro.py:843-844), which does not fit a %dx%d plane" % (C0, C1))
        half, G, S, GM, G16, S16, GM16, hsc = spec
        M = len(pairs)
        mS = int(reg.maxShift)
        mSf, wf = C0 // 2, C0
        se = int(GM.shape[0])
        terms = self.tensor("terms", (4 * N + 1, wf, wf), torch.float32)
        xw = max(self.lib.zr_xcorr_work_bytes(1, C1, mSf),
                 min(XCORR_WORK, self.lib.zr_xcorr_work_bytes(max(M, 1), C1, mSf)))
        xptr = self.ptr("xcwork", xw)
        if half:
            self.call("D_frame_terms", "zr_xcorr_terms_half", G16.data_ptr(), S16.data_ptr(), GM16.data_ptr(),
                      hsc.data_ptr(), N, C0, C1, mSf, terms.data_ptr(), xptr, xw, st)
        else:
            self.call("D_frame_terms", "zr_xcorr_terms", G.data_ptr(), S.data_ptr(), GM.data_ptr(), N, C0, C1, mSf,
                      terms.data_ptr(), xptr, xw, st)
        if refine:
            groups = [[k] for k in range(M)]
            npl = max(M, 1)
        else:
            d = pairs[:, 1] - pairs[:, 0]
            groups = [[int(k) for k in np.nonzero(d == v)[0]] for v in np.unique(d)]
            npl = max([len(g) for g in groups] + [1])
        planes = self.tensor("full_planes", (npl, wf, wf), torch.float32)
        filt = self.tensor("full_filt", (npl, wf, wf), torch.float32)
        if refine:
            TG = self.tensor("refineT", (N, se, 2), torch.float32)
            rterms = self.tensor("refine_terms", (4 * N + 1, wf, wf), torch.float32)
            self.call("E_pairs", "zr_refine_spectra", G.data_ptr(), N, C0, C1, TG.data_ptr(), st)
            self.call("E_pairs", "zr_refine_terms", terms.data_ptr(), N, mSf, rterms.data_ptr(), st)
            self.call("E_pairs", "zr_xcorr_refine", G.data_ptr(), TG.data_ptr(), rterms.data_ptr(), N, C0, C1, mSf,
                      planes.data_ptr(), xptr, xw, st)
        fw = self.lib.zr_full_work_bytes(npl, wf)
        fptr = self.ptr("full_work", fw)
        mean = self.tensor("full_mean", (npl,), torch.float32)
        origin = self.tensor("full_origin", (npl,), torch.float32)
        stats = self.tensor("full_stats", (npl, 3), torch.float64)
        taps = self.tensor("full_taps", (npl, 2, 129), torch.float32)
        rad = self.tensor("full_rad", (npl, 2), torch.int32)
        sel = self.tensor("full_sel", (npl,), torch.int32)
        rolls = self.tensor("full_rolls", (npl, 2), torch.int32)
        sig = self.tensor("full_sigma", (npl,), torch.float64)
        nfe = self.tensor("full_nfev", (npl,), torch.int32)
        res = self.tensor("full_res", (npl, C.sizeof(PeakResult)), torch.uint8)
        taps_h = np.zeros((npl, 2, 129), np.float32)
        rad_h = np.zeros((npl, 2), np.int32)
        pr = np.zeros(M, dtype=_PEAK_DTYPE)
        keep = np.zeros(M, dtype=bool)
        sh_un = np.zeros((N, N, 2))
        row_done = set()
        auto = reg.triMode == "auto"
        npx = float(wf) * float(wf)

        def filter_planes(idx, sy, sx, keep_filtered):
            for p, a, b in zip(idx, sy, sx):
                for axis, sg in ((0, a), (1, b)):
                    t, r = hm.gaussian_taps(sg)
                    taps_h[p, axis, :] = 0.0
                    taps_h[p, axis, :t.size] = t
                    rad_h[p, axis] = r
            taps.copy_(torch.from_numpy(taps_h))
            rad.copy_(torch.from_numpy(rad_h))
            sel[:len(idx)].copy_(torch.from_numpy(np.asarray(idx, dtype=np.int32)))
            self.call("F_peaks", "zr_full_filter", planes.data_ptr(), npl, wf, sel.data_ptr(), len(idx),
                      taps.data_ptr(), rad.data_ptr(), mean.data_ptr(),
                      filt.data_ptr() if keep_filtered else None, stats.data_ptr(), fptr, fw, st)

        for g in groups:
            ks = [k for k in g if not (auto and int(pairs[k][0]) in row_done)]
            if not ks:
                continue
            n = len(ks)
            if refine:
                idx = ks
                for k in ks:
                    self.call("F_peaks", "zr_full_prepare", planes[k].data_ptr(), 1, wf, pp.suppress_origin,
                              origin[k:].data_ptr(), mean[k:].data_ptr(), st)
            else:
                idx = list(range(n))
                pd = torch.from_numpy(np.ascontiguousarray(pairs[ks], dtype=np.int32).reshape(-1)).to(self.dev)
                if half:
                    self.call("E_pairs", "zr_xcorr_pairs_half", G16.data_ptr(), hsc.data_ptr(), terms.data_ptr(),
                              pd.data_ptr(), n, N, C0, C1, mSf, planes.data_ptr(), xptr, xw, st)
                else:
                    self.call("E_pairs", "zr_xcorr_pairs", G.data_ptr(), terms.data_ptr(), pd.data_ptr(), n, N, C0,
                              C1, mSf, planes.data_ptr(), xptr, xw, st)
                self.call("F_peaks", "zr_full_prepare", planes.data_ptr(), n, wf, pp.suppress_origin,
                          origin.data_ptr(), mean.data_ptr(), st)
            nf = np.zeros(n, dtype=np.int32)
            sigma = np.full(n, np.nan)
            if pp.bmode == 1:
                gens = [hm.brent_bounded(pp.opti_lo, pp.opti_hi, pp.opti_xatol, pp.opti_maxiter) for _ in ks]
                xs = [next(gn) for gn in gens]
                act = list(range(n))
                while act:
                    filter_planes([idx[i] for i in act], [xs[i] for i in act], [xs[i] for i in act], False)
                    sth = stats.cpu().numpy()
                    mh = mean.cpu().numpy().astype(np.float64)
                    nxt = []
                    for i in act:
                        s1, s2, mx = sth[idx[i]]
                        m1 = s1 / npx
                        var = s2 / npx - m1 * m1
                        with np.errstate(all="ignore"):
                            f = float(np.float64(math.sqrt(var if var > 0.0 else 0.0)) / np.float64(mx - (mh[idx[i]] + m1)))
                        try:
                            xs[i] = gens[i].send(f)
                            nxt.append(i)
                        except StopIteration as stop:
                            sigma[i], nf[i] = stop.value
                    act = nxt
                sy = sx = list(sigma)
            elif pp.bmode == 2:
                sy, sx = [pp.conv_sigma_y] * n, [pp.conv_sigma_x] * n
            else:
                sy = sx = [0.0] * n
            filter_planes(idx, sy, sx, True)
            rolls_h = np.zeros((npl, 2), np.int32)
            sig_h = np.full(npl, np.nan)
            nf_h = np.zeros(npl, np.int32)
            for i, k in enumerate(ks):
                I, J = int(pairs[k][0]), int(pairs[k][1])
                prev = sh_un[I - 1, I - 1] if refine else sh_un[I, J - 1]
                rolls_h[idx[i]] = np.round(prev).astype(np.int32)
                sig_h[idx[i]] = sigma[i]
                nf_h[idx[i]] = nf[i]
            rolls.copy_(torch.from_numpy(rolls_h))
            sig.copy_(torch.from_numpy(sig_h))
            nfe.copy_(torch.from_numpy(nf_h))
            self.call("F_peaks", "zr_full_peaks", planes.data_ptr(), filt.data_ptr(), npl, wf, sel.data_ptr(), n, mS,
                      rolls.data_ptr(), mean.data_ptr(), origin.data_ptr(), sig.data_ptr(), nfe.data_ptr(),
                      pp.sub_pix_reg, res.data_ptr(), fptr, fw, st)
            recs = np.frombuffer(res.cpu().numpy().tobytes(), dtype=_PEAK_DTYPE)
            for i, k in enumerate(ks):
                r = recs[idx[i]]
                pr[k] = r
                keep[k] = True
                I, J = int(pairs[k][0]), int(pairs[k][1])
                sh_un[I, J] = (r["sy"], r["sx"])
                if auto and (r["peaksig"] <= reg.peaksigThres or J - I >= reg.autoMax):
                    row_done.add(I)
        return pr, keep

    def _align(self, reg):
        """One movie: prepare, correlate, solve, shift, filter, FRC."""
        job = self._prepare(reg)
        self._correlate([job])
        return self._finish(job)

    def _prepare(self, reg, pfx=""):
        """Upload, Fourier binning, hot-pixel filter, padded and crop sizes,
        mask and per-frame mean of one movie.  Returns the movie's job state;
        ``pfx`` keeps its buffers apart from the other movies of a batch."""
        torch = self.torch
        st = self.stream
        bench = {}
        bench["align0"] = time.time()
        if reg.shiftMethod == "fourier":
            # the reference stops in xcorrnm2_tri while storing the full spectra
            # that shift method needs (self.__sC2 is undefined, zorro.py:891-895)
            raise AttributeError("shiftMethod 'fourier' is broken in the reference: self.__sC2 is undefined "
                                 "(zorro.py:895)")
        raw, gain, rtype = self.upload(reg, pfx)
        N, H, W = (int(s) for s in raw.shape)
        raw_float = bool(getattr(reg, "imagesAreRaw", False))
        gdiv = float(reg.gain) if (reg.gain and not np.isclose(reg.gain, 1.0) and (rtype != _lib.ZR_F32 or raw_float)) \
            else 0.0
        frames = self._frames(raw, rtype, gain, gdiv=gdiv)
        pixelsize = reg.pixelsize
        if reg.shapeBinned is not None and np.any(reg.shapeBinned):
            # binStack (zorro.py:1826-1904), before the hot-pixel filter as there
            Hb, Wb = int(reg.shapeBinned[0]), int(reg.shapeBinned[1])
            bwb = self.lib.zr_bin_work_bytes(H, W, Hb, Wb)
            binned = self.tensor(pfx + "binned", (N, Hb, Wb), torch.float32)
            self.call("A_gain_sum", "zr_bin_fourier", C.byref(frames), Hb, Wb, binned.data_ptr(),
                      self.ptr(pfx + "binwork", bwb), bwb, st)
            scale = np.array([H, W], dtype=np.float64) / np.array([Hb, Wb], dtype=np.float64)
            if pixelsize is not None:
                pixelsize = pixelsize * np.mean(scale)
            raw, gain, rtype, gdiv = binned, None, _lib.ZR_F32, 0.0
            N, H, W = (int(v) for v in binned.shape)
            frames = self._frames(raw, rtype, gain)
        hotinfo = dict(reg.hotpixInfo)
        filt = [f for f in (reg.filterMode or "").lower().replace(" ", "").split(",") if f]

        # ---- hot pixels (zorro.py:2497-2672)
        ha = hb = None
        hot_counts = None
        if "hot" in filt:
            bench["hot0"] = time.time()
            usum = self.tensor(pfx + "usum", (H, W), torch.float32)
            tot = self.tensor(pfx + "tot", (4,), torch.float64)
            tot.zero_()
            self.call("A_gain_sum", "zr_gain_sum", C.byref(frames), usum.data_ptr(), tot.data_ptr(), st)
            sumMean, pstd, edges = hm.hotpix_bins(float(tot[0].item()) / (H * W), hotinfo["maxSigma"])
            nb = len(edges) - 1
            hist = self.tensor(pfx + "hist", (nb + 4,), torch.int32)
            hist.zero_()
            self.call("A_gain_sum", "zr_histogram", usum.data_ptr(), H * W, float(edges[0]), nb, hist.data_ptr(), st)
            h = hist[:nb].cpu().numpy().astype(np.int64)
            t_fit = time.perf_counter()
            mu, sg, cl, cu, info = hm.hotpix_fit(h, edges, sumMean, pstd, hotinfo)
            self._host_time("hotpix_fit", t_fit)
            hotinfo.update(info)
            prm = HotpixParams()
            prm.mu, prm.sigma = float(mu), float(sg)
            prm.cutoff_lower, prm.cutoff_upper = float(cl), float(cu)
            prm.logistic_k, prm.relax = float(np.float32(hotinfo["logisticK"])), float(np.float32(hotinfo["relax"]))
            psf = hm.psf_kernel(hotinfo.get("psf", "K2")).ravel()
            for i in range(9):
                prm.psf[i] = float(psf[i])
            prm.neighbour_thres = 0.01
            prm.best_mean = float(mu / N)
            ha = self.tensor(pfx + "hot_a", (H, W), torch.float32)
            hb = self.tensor(pfx + "hot_b", (H, W), torch.float32)
            cnt = self.tensor(pfx + "hotcnt", (4,), torch.int32)
            cnt.zero_()
            wb = self.lib.zr_hotpix_work_bytes(H, W)
            self.call("B_hot_maps", "zr_hotpix_maps", usum.data_ptr(), H, W, N, C.byref(prm), ha.data_ptr(), hb.data_ptr(),
                      cnt.data_ptr(), self.ptr(pfx + "hotwork", wb), wb, st)
            # the dead, hot and neighbour counts are only reported: they are
            # read once the peaks are on the host, so no synchronisation holds
            # back the spectra (the keys keep their place in hotpixInfo)
            hot_counts = cnt
            hotinfo["guessDeadpix"] = hotinfo["guessHotpix"] = hotinfo["neighborPix"] = None
            hotinfo["frameMean"] = float(mu / N)
            hotinfo["frameStd"] = float(sg / np.sqrt(N))
            frames = self._frames(raw, rtype, gain, ha, hb, gdiv)
            bench["hot1"] = time.time()
        hook = getattr(self._tls, "after_hot", None)
        if hook is not None:
            self._tls.after_hot = None
            hook()

        # ---- padding and crop sizes (padStack zorro.py:1908, __init_xcorrnm2 zorro.py:598-611)
        if reg.shapePadded is not None and np.any(reg.shapePadded):
            P0, P1 = int(reg.shapePadded[0]), int(reg.shapePadded[1])
        else:
            P0, P1 = H, W
        if H > P0 or W > P1:
            raise ValueError("shapePadded %s is smaller than the frames %s" % ([P0, P1], [H, W]))
        if reg.fouCrop is not None and np.any(reg.fouCrop):
            C0, C1 = (int(v) for v in 2 * np.floor(np.array(reg.fouCrop) / 2.0).astype(int))
        else:
            C0, C1 = P0, P1
        for v, nm, ok in ((P0, "shapePadded", _PADDED_OK), (P1, "shapePadded", _PADDED_OK), (C0, "fouCrop", _CROP_OK),
                          (C1, "fouCrop", _CROP_OK)):
            if not ok(v):
                raise ValueError("%s %d: the GPU path transforms powers of two (64..4096) and 1536, 3072, 6144 "
                                 "(padded) or 384, 768, 1536, 3072 (crop)" % (nm, v))
        mS = int(reg.maxShift)
        w = 2 * mS
        if 2 <= mS and 2 * mS <= min(C0, C1):
            self.plan(P0, P1, C0, C1, mS, getattr(reg, "fftw_effort", "FFTW_MEASURE"), getattr(reg, "cachePath", None))
        mask_dev = None
        user_mask = reg.masks is not None and len(np.shape(reg.masks)) > 0
        if user_mask:
            m = np.asarray(reg.masks)
            if m.ndim == 3 and m.shape[0] > 1:
                raise ValueError("per-frame masks are not supported by the GPU path")
            m = m.reshape(m.shape[-2], m.shape[-1]).astype(np.float32)
            mp = np.zeros((P0, P1), np.float32)
            mp[:m.shape[0], :m.shape[1]] = m
            mask_dev = torch.from_numpy(mp).to(self.dev, non_blocking=True)
        msub = None
        if reg.subtractFrameMean and not user_mask:
            msub = self.tensor(pfx + "msub", (N,), torch.float64)
            if "hot" in filt:
                # any per-frame constant is exact; the mean frame of the unaligned
                # sum is close to every frame's mean and costs no extra pass
                msub.copy_(tot[0].expand(N) / N)
            else:
                msub.zero_()
                self.call("C_spectra", "zr_frame_sums", C.byref(frames), msub.data_ptr(), st)
        job = types.SimpleNamespace(
            reg=reg, pfx=pfx, bench=bench, raw=raw, gain=gain, rtype=rtype, gdiv=gdiv, N=N, H=H, W=W, frames=frames,
            pixelsize=pixelsize, hotinfo=hotinfo, filt=filt, ha=ha, hb=hb, P0=P0, P1=P1, C0=C0, C1=C1, mS=mS, w=w,
            mask_dev=mask_dev, user_mask=user_mask, msub=msub, hot_counts=hot_counts,
            half=str(getattr(reg, "spectraPrecision", "float32")).lower() in ("float16", "half", "f16"),
            refine=reg.triMode == "refine", preshift=bool(reg.preShift and mS))
        if job.half and job.refine:
            raise ValueError("triMode 'refine' builds its templates from float32 spectra (spectraPrecision 'float32')")
        if job.refine:
            # frame I against the template of the others, I < N-1 (zorro.py:941-954)
            job.pairs = np.array([(I, I) for I in range(N - 1)], dtype=np.int32).reshape(-1, 2)
        else:
            job.pairs = hm.pair_list(hm.tri_indices(N, reg.triMode, reg.diagWidth, reg.diagStart))
        job.pp = self._peak_params(reg, P0, P1)
        return job

    def _peak_params(self, reg, P0, P1):
        """locatePeak's settings (zorro.py:1099-1231) as zr_peak_params_t."""
        pp = PeakParams()
        pp.sub_pix_reg = int(reg.subPixReg or 1)
        bm = str(reg.Bmode)
        if bm == "opti":
            pp.bmode = 1
        elif reg.Brad and bm in ("conv", "convolution"):
            pp.bmode = 2
            pp.conv_sigma_y = P0 / (np.sqrt(2) * np.pi * reg.Brad)
            pp.conv_sigma_x = P1 / (np.sqrt(2) * np.pi * reg.Brad)
        elif bm == "fourier":
            raise ValueError("Bmode 'fourier' is broken in the reference (normConst undefined, zorro.py:1132)")
        else:
            pp.bmode = 0
        pp.suppress_origin = int(bool(reg.suppressOrigin))
        pp.use_mask = 1
        pp.opti_lo, pp.opti_hi, pp.opti_xatol, pp.opti_maxiter = 0.0, 7.0, 0.01, 15
        return pp

    # ------------------------------------------------------------------ spectra and pairs
    def _correlate(self, jobs, cls=""):
        """Forward spectra, frame terms, correlation windows and peaks
        (xcorrnm2_tri, mnxc2, locatePeak) of one movie, or of several movies
        of one shape class in one set of launches: their frames concatenated
        (each frame reading its own movie's gain and hot-pixel maps), the
        frame terms of all frames, every movie's pairs with its frames'
        offsets, and all windows' peaks.  Sets each job's ``pr`` and ``keep``."""
        for j in jobs:
            j.bench["xcorr0"] = time.time()
        if len(jobs) == 1:
            self._correlate_one(jobs[0])
        else:
            self._correlate_batch(jobs, cls)
        for j in jobs:
            reg = j.reg
            keep = j.keep
            if not j.preshift and reg.triMode == "auto":
                row_done = {}
                for k, (I, J) in enumerate(j.pairs):
                    if row_done.get(I):
                        keep[k] = False
                        continue
                    if j.pr["peaksig"][k] <= reg.peaksigThres or J - I >= reg.autoMax:
                        row_done[I] = True
            j.bench["xcorr2"] = time.time()

    def _spectra_pass(self, frames, mask_dev, msub, N, H, P0, P1, C0, C1, G, S, pfx, half=None):
        """zr_spectra over frames [0, N) in chunks that fit SPECTRA_WORK;
        ``half`` = (G16, S16, hsc, packwork) packs each chunk to half
        precision (G and S are then one chunk long)."""
        st = self.stream
        per = self.lib.zr_spectra_work_bytes(H, 1, C1)
        chunk = max(1, min(N, SPECTRA_WORK // per))
        wb = per * chunk
        wptr = self.ptr(pfx + "specwork", wb)
        se = int(self.lib.zr_spectrum_elems(C0, C1))
        for f0 in range(0, N, chunk):
            nf = min(chunk, N - f0)
            g0 = 0 if half else f0
            self.call("C_spectra", "zr_spectra", C.byref(frames), mask_dev.data_ptr() if mask_dev is not None else None,
                      msub.data_ptr() if msub is not None else None, f0, nf, 0, P0, P1, C0, C1,
                      G[g0].data_ptr(), S[g0].data_ptr(), wptr, wb, st)
            if half:
                G16, S16, hsc, pw = half
                self.call("C_spectra", "zr_pack_half", G.data_ptr(), nf, se, G16[f0].data_ptr(), hsc[f0:].data_ptr(),
                          pw, 4 * N, st)
                self.call("C_spectra", "zr_pack_half", S.data_ptr(), nf, se, S16[f0].data_ptr(),
                          hsc[N + f0:].data_ptr(), pw, 4 * N, st)

    def _mask_spectrum(self, frames, mask_dev, H, P0, P1, C0, C1, pfx):
        torch = self.torch
        se = int(self.lib.zr_spectrum_elems(C0, C1))
        GM = self.tensor(pfx + "GM", (se, 2), torch.float32)
        mrows = P0 if mask_dev is not None else H
        wbm = self.lib.zr_spectra_work_bytes(mrows, 1, C1)
        self.call("C_spectra", "zr_spectra", C.byref(frames), mask_dev.data_ptr() if mask_dev is not None else None,
                  None, 0, 1, 1, P0, P1, C0, C1, GM.data_ptr(), None, self.ptr(pfx + "specwork", wbm), wbm,
                  self.stream)
        return GM

    def _correlate_one(self, job):
        torch = self.torch
        st = self.stream
        reg, pfx = job.reg, job.pfx
        N, H, P0, P1, C0, C1 = job.N, job.H, job.P0, job.P1, job.C0, job.C1
        se = int(self.lib.zr_spectrum_elems(C0, C1))
        per = self.lib.zr_spectra_work_bytes(H, 1, C1)
        chunk = max(1, min(N, SPECTRA_WORK // per))
        half = job.half
        G16 = S16 = GM16 = hsc = None
        if half:
            # half-precision store with per-spectrum power-of-two scales: each
            # chunk of frames goes through a float32 staging buffer, then packed
            G16 = self.tensor(pfx + "G16", (N, se), torch.int32)
            S16 = self.tensor(pfx + "S16", (N, se), torch.int32)
            GM16 = self.tensor(pfx + "GM16", (se,), torch.int32)
            hsc = self.tensor(pfx + "hscales", (2 * N + 1,), torch.float32)
            pw = self.ptr(pfx + "packwork", 4 * max(N, 1))
            G = self.tensor(pfx + "G", (chunk, se, 2), torch.float32)
            S = self.tensor(pfx + "S", (chunk, se, 2), torch.float32)
        else:
            G = self.tensor(pfx + "G", (N, se, 2), torch.float32)
            S = self.tensor(pfx + "S", (N, se, 2), torch.float32)
        GM = self._mask_spectrum(job.frames, job.mask_dev, H, P0, P1, C0, C1, pfx)
        if half:
            self.call("C_spectra", "zr_pack_half", GM.data_ptr(), 1, se, GM16.data_ptr(), hsc[2 * N:].data_ptr(),
                      pw, 4 * N, st)
        self._spectra_pass(job.frames, job.mask_dev, job.msub, N, H, P0, P1, C0, C1, G, S, pfx,
                           half=(G16, S16, hsc, pw) if half else None)
        spec = (half, G, S, GM, G16, S16, GM16, hsc)
        if job.preshift:
            job.pr, job.keep = self._preshift(reg, job.pairs, job.refine, N, C0, C1, job.pp, spec, st)
        else:
            job.pr = self._cropped_peaks(reg, job.pairs, job.refine, N, C0, C1, job.mS, job.pp, spec, st)
            job.keep = np.ones(len(job.pairs), dtype=bool)

    @staticmethod
    def batch_key(job):
        """Movies with equal keys share the launches of the batched path: the
        same frame shape and pixel type, the same corrections, transform
        sizes and peak search.  None: the movie goes alone (preShift,
        triMode 'refine', half-precision spectra, a user mask)."""
        if job.preshift or job.refine or job.half or job.user_mask:
            return None
        r = job.reg
        pp = job.pp
        return (job.H, job.W, job.rtype, job.gain is not None, job.ha is not None, job.gdiv, job.msub is not None,
                job.P0, job.P1, job.C0, job.C1, job.mS, pp.bmode, pp.sub_pix_reg, pp.suppress_origin,
                pp.conv_sigma_y, pp.conv_sigma_x, bool(r.subtractFrameMean))

    def _correlate_batch(self, jobs, cls):
        torch = self.torch
        st = self.stream
        j0 = jobs[0]
        H, W, P0, P1, C0, C1, mS = j0.H, j0.W, j0.P0, j0.P1, j0.C0, j0.C1, j0.mS
        w = 2 * mS
        pfx = cls
        Ns = [j.N for j in jobs]
        offs = np.concatenate([[0], np.cumsum(Ns)]).astype(np.int64)
        NT = int(offs[-1])
        HW = H * W
        # the movies' frames and maps side by side (device copies)
        tdt = j0.raw.dtype
        raw = self.tensor(pfx + "raw", (NT, H, W), tdt)
        for j, f0 in zip(jobs, offs):
            raw[int(f0):int(f0) + j.N].copy_(j.raw)

        def stacked(name, attr):
            if getattr(j0, attr) is None:
                return None
            t = self.tensor(pfx + name, (len(jobs), H, W), torch.float32)
            for k, j in enumerate(jobs):
                t[k].copy_(getattr(j, attr).reshape(H, W))
            return t
        gain, ha, hb = stacked("gain", "gain"), stacked("hot_a", "ha"), stacked("hot_b", "hb")
        fmap = torch.from_numpy(np.repeat(np.arange(len(jobs), dtype=np.int32), Ns)).to(self.dev, non_blocking=True)
        frames = Frames(raw.data_ptr(), j0.rtype, gain.data_ptr() if gain is not None else None,
                        ha.data_ptr() if ha is not None else None, hb.data_ptr() if hb is not None else None,
                        float(j0.gdiv), NT, H, W, HW, fmap.data_ptr(), HW)
        msub = None
        if j0.msub is not None:
            msub = self.tensor(pfx + "msub", (NT,), torch.float64)
            for j, f0 in zip(jobs, offs):
                msub[int(f0):int(f0) + j.N].copy_(j.msub)
        se = int(self.lib.zr_spectrum_elems(C0, C1))
        G = self.tensor(pfx + "G", (NT, se, 2), torch.float32)
        S = self.tensor(pfx + "S", (NT, se, 2), torch.float32)
        GM = self._mask_spectrum(j0.frames, None, H, P0, P1, C0, C1, pfx)
        self._spectra_pass(frames, None, msub, NT, H, P0, P1, C0, C1, G, S, pfx)
        # frame terms of every frame, then every movie's pairs at its frames' offsets
        terms = self.tensor(pfx + "terms", (4 * NT + 1, w, w), torch.float32)
        pairs = np.concatenate([j.pairs + int(f0) for j, f0 in zip(jobs, offs)]).astype(np.int32)
        M = len(pairs)
        xw = min(XCORR_WORK, max(self.lib.zr_xcorr_work_bytes(1, C1, mS), self.lib.zr_xcorr_work_bytes(M, C1, mS)))
        xptr = self.ptr(pfx + "xcwork", xw)
        self.call("D_frame_terms", "zr_xcorr_terms", G.data_ptr(), S.data_ptr(), GM.data_ptr(), NT, C0, C1, mS,
                  terms.data_ptr(), xptr, xw, st)
        cwin = self.tensor(pfx + "cwin", (max(M, 1), w, w), torch.float32)
        pairs_dev = torch.from_numpy(pairs.reshape(-1)).to(self.dev, non_blocking=True)
        self.call("E_pairs", "zr_xcorr_pairs", G.data_ptr(), terms.data_ptr(), pairs_dev.data_ptr(), M, NT, C0, C1,
                  mS, cwin.data_ptr(), xptr, xw, st)
        pres = self.tensor(pfx + "peaks", (max(M, 1), C.sizeof(PeakResult)), torch.uint8)
        self.call("F_peaks", "zr_locate_peaks", cwin.data_ptr(), M, mS, C.byref(j0.pp), pres.data_ptr(), st)
        recs = np.frombuffer(pres[:M].cpu().numpy().tobytes(), dtype=_PEAK_DTYPE).copy()
        k = 0
        for j in jobs:
            m = len(j.pairs)
            j.pr = recs[k:k + m].copy()
            j.keep = np.ones(m, dtype=bool)
            k += m

    # ------------------------------------------------------------------ solve, shifts, filters, FRC
    def _finish(self, job):
        """The drift solve, shifted sums, dose filter, FRC and outputs of one
        movie."""
        return self._finish_out(job, self._finish_main(job))

    def _finish_main(self, job):
        """The drift solve, the shifted sums and the dose filter of one movie
        (zorro.py:1651-1712); keeps what the FRC and the outputs need on the
        job and returns the outputs so far."""
        torch = self.torch
        st = self.stream
        reg, pfx, bench = job.reg, job.pfx, job.bench
        N, H, W, P0, P1, C0, C1 = job.N, job.H, job.W, job.P0, job.P1, job.C0, job.C1
        pairs, pr, keep = job.pairs, job.pr, job.keep
        filt, hotinfo, frames, pixelsize, user_mask = job.filt, job.hotinfo, job.frames, job.pixelsize, job.user_mask
        refine = job.refine
        if job.hot_counts is not None:  # complete: the peaks came back after them on this stream
            c = job.hot_counts.cpu().numpy()
            hotinfo["guessDeadpix"], hotinfo["guessHotpix"], hotinfo["neighborPix"] = int(c[0]), int(c[1]), int(c[2])
            job.hot_counts = None
        shifts = np.zeros([N, N, 2])
        corr = np.zeros([N, N])
        psig = np.zeros([N, N])
        orig = np.zeros([N, N])
        Ii, Jj = pairs[keep, 0], pairs[keep, 1]
        shifts[Ii, Jj, 0] = pr["sy"][keep]
        shifts[Ii, Jj, 1] = pr["sx"][keep]
        corr[Ii, Jj] = pr["corr"][keep]
        psig[Ii, Jj] = pr["peaksig"][keep]
        orig[Ii, Jj] = pr["origin"][keep]
        if reg.fouCrop is not None and np.any(reg.fouCrop):
            shifts[:, :, 0] *= P0 / C0
            shifts[:, :, 1] *= P1 / C1
        self.last_peaks = pr
        self.last_pairs = pairs
        bench["xcorr3"] = time.time()

        # ---- drift solve (shiftsSolver zorro.py:1260-1567)
        out = {}
        edl = list(reg.errorDictList)
        finish_errors = None
        if reg.triMode == "first":
            translations = -shifts[0, :]
            ed = {"shiftsTriMat": shifts, "corrTriMat": corr, "originTriMat": orig, "peaksigTriMat": psig,
                  "translations": translations.copy()}
        elif refine:
            # zorro.py:1635-1647: the negated diagonal, in a float32 array
            translations = np.zeros([N, 2], dtype="float32")
            for K in range(N):
                translations[K, :] = -shifts[K, K, :]
            ed = {"shiftsTriMat": shifts, "corrTriMat": corr, "originTriMat": orig, "peaksigTriMat": psig,
                  "translations": translations.copy()}
        else:
            t_solve = time.perf_counter()
            # the error analysis of the solve waits until the shifted sums are
            # queued (finish_errors below): only the translations gate them
            ed, trans, finish_errors = hm.solve_shifts(
                shifts, corr, psig, shapeImage=[P0, P1], maxShift=reg.maxShift, weightMode=reg.weightMode,
                peaksigThres=reg.peaksigThres, logisticK=reg.logisticK, logisticNu=reg.logisticNu, defer_errors=True)
            self._host_time("drift_solve", t_solve)
            if reg.weightMode == "autologistic":
                out["peaksigThres"] = ed["peaksigThres"]
                out["logisticK"] = ed["logisticK"]
                out["logisticNu"] = ed["logisticNu"]
            translations = trans.copy()
        edl.append(ed)
        out["errorDictList"] = edl
        bench["solve1"] = time.time()

        # ---- shifts and sums (applyShifts zorro.py:1734-1808)
        if reg.originMode == "centroid":
            translations = translations - np.mean(translations, axis=0)
        # integer roll only unless subPixReg > 1 with 'lanczos' (zorro.py:1790-1796)
        tab = hm.shift_table(translations, H, W, lanczos=reg.subPixReg > 1.0 and reg.shiftMethod == "lanczos")
        sh_dev = torch.from_numpy(tab.view(np.uint8)).to(self.dev, non_blocking=True)
        isum = self.tensor(pfx + "isum", (H, W), torch.float32)
        # the even/odd half sums feed only the lazy FRC (the independent
        # even/odd FRC registers the halves again)
        lazy = bool(reg.doLazyFRC) and not reg.doEvenOddFRC
        esum = self.tensor(pfx + "esum", (H, W), torch.float32) if lazy else None
        osum = self.tensor(pfx + "osum", (H, W), torch.float32) if lazy else None
        need_aligned = (reg.keepAlignedImages or bool(reg.doEvenOddFRC) or
                        any(f in ("dose", "dosenorm") for f in filt))
        aligned = self.tensor(pfx + "aligned", (N, H, W), torch.float32) if need_aligned else None
        self.call("G_shift_sum", "zr_shift_sum", C.byref(frames), sh_dev.data_ptr(), isum.data_ptr(),
                  esum.data_ptr() if lazy else None, osum.data_ptr() if lazy else None,
                  aligned.data_ptr() if aligned is not None else None, st)
        bench["shifts1"] = time.time()

        # the aligned stack is complete here: the half-set registrations of the
        # even/odd FRC wait on this event, not on the stream, so that the dose
        # filter below runs on the GPU while they do their host steps
        aligned_ready = torch.cuda.Event()
        aligned_ready.record()

        # ---- dose filter (zorro.py:2349-2494)
        filt_sum = None
        for fm in filt:
            if fm in ("dose", "dosenorm"):
                mean_sum = float(isum.double().mean().item()) if reg.doseFiltParam[0] is None else None
                dc = hm.dose_constants(N, [P0, P1], pixelsize, reg.voltage, reg.doseFiltParam, mean_sum)
                dp = DoseParams(dc["A"], dc["B"], dc["C"], dc["order"], dc["vs"], dc["invPSx"], dc["invPSy"],
                                int(fm == "dosenorm"))
                tq = torch.from_numpy(dc["thresQ"].astype(np.float32)).to(self.dev, non_blocking=True)
                de = torch.from_numpy(dc["dose_end"].astype(np.float32)).to(self.dev, non_blocking=True)
                fixed = self.lib.zr_dose_work_bytes(P0, P1, 0)
                perf = self.lib.zr_dose_work_bytes(P0, P1, 1) - fixed
                nch = max(2, min(N + (N & 1), (DOSE_WORK - fixed) // perf))
                dwb = fixed + nch * perf
                filt_sum = self.tensor(pfx + "filtsum", (H, W), torch.float32)
                self.call("I_dose", "zr_dose_filter", aligned.data_ptr(), N, H, W, C.byref(dp), tq.data_ptr(), de.data_ptr(),
                          P0, P1, filt_sum.data_ptr(), self.ptr(pfx + "dosework", dwb), dwb, st)
        bench["dose1"] = time.time()
        # host results: the sums are final now, so their copies to pinned host
        # memory go on a side stream at once, behind the kernels that make
        # them, and overlap what follows (the half-set registrations)
        early = {}
        if not bool(getattr(reg, "returnDeviceArrays", False)):
            made = torch.cuda.Event()
            made.record()
            side = self._copy_stream()
            side.wait_event(made)
            with torch.cuda.stream(side):
                for k, t in (("imageSum", isum), ("filtSum", filt_sum)):
                    if t is not None:
                        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
                        h.copy_(t, non_blocking=True)
                        early[k] = h
            if early:
                copied = torch.cuda.Event()
                copied.record(side)
                early[None] = copied
        job.early = early
        if finish_errors is not None:  # while the GPU shifts, sums and filters
            finish_errors()
            ed["originTriMat"] = orig

        job.translations, job.isum, job.esum, job.osum = translations, isum, esum, osum
        job.aligned, job.aligned_ready, job.filt_sum = aligned, aligned_ready, filt_sum
        return out

    def _finish_out(self, job, out, halves=None):
        """FRC (lazy, or the independent even/odd FRC) and the outputs of one
        movie.  ``halves``: (FRC, FRC2D, transEven, transOdd, half-set error
        dictionaries) when the batched path has registered the half sets."""
        torch = self.torch
        st = self.stream
        reg, pfx, bench = job.reg, job.pfx, job.bench
        H, W, N = job.H, job.W, job.N
        hotinfo, filt, pixelsize, user_mask = job.hotinfo, job.filt, job.pixelsize, job.user_mask
        translations, isum, esum, osum = job.translations, job.isum, job.esum, job.osum
        aligned, filt_sum = job.aligned, job.filt_sum
        # ---- lazy FRC (zorro.py:2226-2310)
        frc = frc2d = None
        if reg.doEvenOddFRC:
            if halves is None:
                halves = self._even_odd_frc(reg, aligned, hotinfo, filt, job.aligned_ready)
            frc, frc2d, out["transEven"], out["transOdd"], out["halfSetErrorDicts"] = halves
        elif reg.doLazyFRC:
            offs, tiles = hm.frc_tiles((H, W), translations)
            box = 512
            if len(offs) and (offs.min() < 0 or (offs[:, 0] + box).max() > H or (offs[:, 1] + box).max() > W):
                raise ValueError("tiledFRC: tiles %s leave the %dx%d image (negative crop limits)" % (tiles, H, W))
            if len(offs) == 0:
                frc = np.full(box // 2, np.nan)
                frc2d = np.full((box, box), np.nan, dtype=np.float32)
            else:
                offs_dev = torch.from_numpy(offs.reshape(-1)).to(self.dev, non_blocking=True)
                nr = box // 2
                fwb = self.lib.zr_frc_work_bytes(len(offs), box)
                f2 = self.tensor(pfx + "frc2d", (box, box), torch.float32)
                fr = self.tensor(pfx + "frc", (nr,), torch.float64)
                self.call("H_frc", "zr_tiled_frc", esum.data_ptr(), osum.data_ptr(), H, W, box, offs_dev.data_ptr(), len(offs),
                          f2.data_ptr(), fr.data_ptr(), nr, self.ptr(pfx + "frcwork", fwb), fwb, st)
                frc2d, frc = f2, fr
        bench["frc1"] = time.time()


        # ---- results back to the host (or left on the device)
        out["translations"] = translations
        dev_out = bool(getattr(reg, "returnDeviceArrays", False))

        # host results go through pinned buffers from torch's caching host
        # allocator: all copies are queued on the stream, then one wait; each
        # returned array keeps its pinned block alive
        pending = []

        def fetch(t):
            if isinstance(t, np.ndarray):
                return t
            if dev_out:
                return t.clone()
            h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
            h.copy_(t, non_blocking=True)
            pending.append(h)
            return h

        early = getattr(job, "early", None) or {}
        if early:
            torch.cuda.current_stream(self.dev).wait_event(early[None])
            pending.extend(v for k, v in early.items() if k is not None)
        out["imageSum"] = early["imageSum"] if "imageSum" in early else fetch(isum)
        if frc is not None:
            out["FRC"] = fetch(frc)
            out["FRC2D"] = fetch(frc2d)
        if filt_sum is not None:
            out["filtSum"] = early["filtSum"] if "filtSum" in early else fetch(filt_sum)
        if reg.keepAlignedImages:
            out["images"] = fetch(aligned)
            out["imagesAreRaw"] = False
        if pending:
            torch.cuda.current_stream(self.dev).synchronize()
            for k in ("imageSum", "FRC", "FRC2D", "filtSum", "images"):
                if k in out and isinstance(out[k], torch.Tensor):
                    out[k] = out[k].numpy()
        out["hotpixInfo"] = hotinfo
        out["shapeOriginal"] = [H, W]
        out["pixelsize"] = pixelsize
        if user_mask:
            out["masks"] = reg.masks
        else:
            out["_ones_mask_shape"] = (H, W)  # the all-true mask, made when the registrator's masks are read
        bench["align1"] = time.time()
        b = dict(reg.bench)
        b.update(bench)
        out["bench"] = b
        return out

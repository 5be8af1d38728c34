#!/usr/bin/env python3
"""Movie-registration benchmark: K2-size movies through alignImageStack.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (the K2 configuration): 40 frames of 3838 x 3710 uint8 counts
(Poisson mean 0.8 e/px/frame) with a U(0.9, 1.1) float32 gain map and 0.01 %
hot pixels at 50x the mean, random-walk drift 1.2 px/frame; padded to 4096,
Fourier-cropped to 2048 for the all-pairs triangle (780 pairs, maxShift 100),
hot-pixel filter, Lanczos shift and sum, the independent even/odd FRC (the
even and the odd frames registered again, their sums aligned, tiled FRC)
and the dose filter at 1.2 e/A^2/frame, 1.05 A/px.  Inputs are seeded synthetic movies.

One step registers one movie.  ``value`` is movies/s with the raw frames
already resident in HBM; ``e2e`` is the same through the public API from
pinned host memory (frames and gain copied in, sums, FRC and trajectory
copied out, every step).  The input (570 MB of frames) is larger than L2.
``e2e_packed4`` repeats ``e2e`` with the counts clipped to 15 and packed
two pixels a byte (the MRC mode-101 layout of counting detectors), expanded
on the GPU, and reports the unpack kernel's bandwidth.
Under torchrun each rank registers its own movies (replicas, no collective
on the data path); ``value`` is the job total.

``--impl reference`` times the reference's algorithm on the host cores: the
float32 CPU restatement of the same pipeline (NumPy/SciPy; scipy.fft on every
core stands in for pyFFTW's threaded FFTW plans).  The host work of one
movie is a list of units (hot-pixel filters, per-frame spectra, pairs, drift
solves, per-frame shifts and dose-filter frames, FRC); step k times units k,
k + K, k + 2K, ... so that the K timed steps together measure one whole movie.
The GPU arm's ``cpu_baseline`` times a stratified sample of the same list and
scales it to the movie; the reference arm reports that estimate beside its
measurement.  ``accuracy`` compares the last timed movie with the float64
oracle's outputs for the same seeded movie (tests/golden/oracle_<workload>.npz).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from zorro_gb300.workloads import WORKLOADS  # noqa: E402  (named synthetic workloads)

METRIC = "4k x 4k x 40 movies/sec (K2 3838x3710x40 registration)"

UNIT = "movies/s"


def workload_config(name, world=1):
    """The bench line's ``config``: the workload named by what it is, the
    same object in both arms."""
    wl = WORKLOADS[name]
    mv, at = wl["movie"], wl["attrs"]
    N, (H, W) = mv["n_frames"], mv["shape"]
    pairs = N * (N - 1) // 2 if at["triMode"] == "tri" else None
    desc = "%s: %dx%dx%d %s%s%s, P=%d, C=%d, %s%s, maxShift %d, %s filters" % (
        name, N, H, W, "u8" if mv.get("dtype") == "uint8" else "f32", " + gain" if mv.get("gain_map") else "",
        " + %g%% hot px" % (100 * mv["hot_fraction"]) if mv.get("hot_fraction") else "", at["shapePadded"][0],
        at["fouCrop"][0], at["triMode"], " %d pairs" % pairs if pairs else "", at["maxShift"],
        "+".join(at["filterMode"].split(",")))
    if at.get("doEvenOddFRC"):
        desc += ", even/odd FRC (two half-set registrations of %d frames)" % (N // 2)
    mb = N * H * W * (1 if mv.get("dtype") == "uint8" else 4) / 1e6
    l2 = ("inputs (%d MB raw frames per movie) larger than L2; no flush" % mb if mb > 129 else
          "inputs (%d MB raw frames per movie) smaller than L2: a test workload, not a bench figure" % mb)
    return {"workload": desc, "l2": l2, "parallelism": "replicas" if world > 1 else "single"}


def algorithmic_bytes(N, H, W, C, w, M, b_in, evenodd=False, hot=True):
    """Unique logical bytes per movie and stage: every input element read once,
    every output written once (FFT intermediates excluded).  With ``evenodd``
    the two half-set registrations of the independent FRC (n = N/2 aligned
    float32 frames each, hot filter, spectra, terms, the half triangle,
    shift-sum) and the 'first' alignment of the two sums (with its own hot
    filter) are added to the stages they run in."""
    HW = H * W
    spec = C * (C // 2 + 1) * 8

    def one(n, m, b, hotpix):
        return {"A_gain_sum": (n * HW * b + 8 * HW) if hotpix else 0, "B_hot_maps": 12 * HW if hotpix else 0,
                "C_spectra": n * HW * b + 12 * HW + 2 * n * spec, "D_frame_terms": 2 * n * spec + 16 * n * w * w,
                "E_pairs": n * spec + 4 * m * w * w, "F_peaks": 4 * m * w * w, "G_shift_sum": n * HW * b + 24 * HW}
    ab = one(N, M, b_in, True)
    ab["H_frc"] = 8 * HW
    ab["I_dose"] = N * HW * b_in + 16 * HW
    if evenodd:
        n = N // 2
        for part in (one(n, n * (n - 1) // 2, 4, hot), one(n, n * (n - 1) // 2, 4, hot), one(2, 1, 4, hot)):
            for k, v in part.items():
                ab[k] += v
    return ab


def fft_flops(N, P, C, w, M, evenodd=False):
    """Nominal FFT FLOPs per movie and stage, 5 n log2(n) per complex
    transform of n points (a real transform counts half).  A pruned inverse
    (columns at C, then only the w kept rows) costs (C/2 + 1 + w/2) column/row
    transforms of length C.  ``evenodd`` adds the half-set registrations."""
    import math
    full_real = 2.5 * P * P * math.log2(P * P)
    pruned = (C // 2 + 1 + w // 2) * 5.0 * C * math.log2(C)
    fl = {"C_spectra": 2 * N * full_real, "D_frame_terms": (4 * N + 1) * pruned, "E_pairs": M * pruned,
          "I_dose": (N + 1) * full_real}
    if evenodd:
        n = N // 2
        fl["C_spectra"] += 2 * (2 * n * full_real) + 2 * 2 * full_real
        fl["D_frame_terms"] += 2 * (4 * n + 1) * pruned + 9 * pruned
        fl["E_pairs"] += 2 * (n * (n - 1) // 2) * pruned + pruned
    return fl


def read_traffic():
    """DRAM bytes per movie and stage measured by ncu (profiles/traffic.txt:
    lines '<stage> <bytes>'), or {} when absent."""
    out = {}
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.txt")) as fh:
            for ln in fh:
                p = ln.split("#", 1)[0].split()
                if len(p) >= 2:
                    out[p[0]] = int(float(p[1]))
    except OSError:
        pass
    return out


def movie_timeline(eng, torch, run):
    """One more movie, outside the timed region, with every stage call
    bracketed by CUDA events and the host steps stamped: the movie's time,
    the union of the stage calls' device intervals (GPU busy), and the idle
    gaps with the host steps that overlapped them.  Device and host times
    share a base: an event recorded on an idle GPU at a known host time."""
    import time as _t
    eng.profile = {}
    torch.cuda.synchronize()
    base = torch.cuda.Event(enable_timing=True)
    base.record()
    torch.cuda.synchronize()
    t0 = _t.perf_counter()
    run()
    end = torch.cuda.Event(enable_timing=True)
    end.record()
    torch.cuda.synchronize()
    prof, hosts = eng.profile, eng.host_intervals()
    eng.profile = None
    ivs = sorted((base.elapsed_time(a), base.elapsed_time(b)) for k, v in prof.items()
                 if not k.startswith("host:") for a, b in v)
    busy = []
    for a, b in ivs:
        if busy and a <= busy[-1][1]:
            busy[-1][1] = max(busy[-1][1], b)
        else:
            busy.append([a, b])
    total = base.elapsed_time(end)
    hs = [(k, (a - t0) * 1e3, (b - t0) * 1e3) for k, a, b in hosts]
    gaps, prev = [], 0.0
    for a, b in busy + [[total, total]]:
        if a - prev > 0.1:
            during = sorted({k for k, ha, hb in hs if ha < a and hb > prev})
            gaps.append({"from_ms": round(prev, 2), "ms": round(a - prev, 2), "host": during})
        prev = max(prev, b)
    busy_ms = sum(b - a for a, b in busy)
    idle_host = {}
    for g in gaps:
        key = "+".join(g["host"]) or "launch/sync"
        idle_host[key] = round(idle_host.get(key, 0.0) + g["ms"], 2)
    return {"movie_ms": round(total, 2), "gpu_busy_ms": round(busy_ms, 2), "gpu_idle_ms": round(total - busy_ms, 2),
            "idle_ms_by_host_step": idle_host,
            "host_steps": [{"step": k, "from_ms": round(a, 2), "ms": round(b - a, 2)} for k, a, b in hs],
            "gaps_over_0.1ms": gaps}


def slowest_rank(t_local, dist=None, device="cpu"):
    """Seconds per step of the job: the maximum over ranks of each rank's
    own time (each rank registers its own movies; no data-path collective)."""
    if dist is None:
        return float(t_local)
    import torch
    tt = torch.tensor([float(t_local)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------- CPU baseline

class HostMovieWork:
    """Every unit of host work of one registration of a workload, run by the
    float32 CPU restatement of the reference's algorithm (``oracle``, the
    reference's native complex64/float32; ``scipy.fft`` with ``workers``
    threads stands in for pyFFTW's threaded FFTW plans, NumPy for numexprz).

    A unit is one of: the hot-pixel filter of a whole stack (with its CDF fit
    and its per-pixel neighbour loop), the forward spectra of one frame, one
    pair (mnxc2 and locatePeak), one drift solve, the shift of one frame, one
    frame of the dose filter (plus its set-up and final inverse), one tiled
    FRC.  With the even/odd FRC the list also holds the two half-set
    registrations (their own hot-pixel filter, spectra, pairs, solve and
    shifts) and the 'first' alignment of the two half sums.  Units of the same
    kind cost the same whatever frame they touch, so spectra, pairs, shifts
    and dose frames run on fixed frames; the hot-pixel filters run on the
    stacks they see in the pipeline (the raw-derived stack, the aligned half
    sets, the pair of half sums) because their neighbour loop depends on the
    content."""

    # units timed by the stratified sample of one movie: every STRIDE-th unit
    # of each stratum (the first always), scaled by the stratum's count; a
    # stratum is a kind of unit within the movie, the two half sets together,
    # or the pair of half sums
    STRIDE = {"spectra": 10, "pair": 40, "shift": 10, "dose_frame": 10, "hot": 2}

    @staticmethod
    def stratum(unit):
        tag, kind, _ = unit
        return ("half" if tag in ("even", "odd") else tag, kind)

    def __init__(self, mv, attrs, workers):
        from oracle import zorro_oracle as zo
        self.zo = zo
        self.attrs = attrs
        self.dt = zo.Dtypes(False, workers)
        imgs = np.ascontiguousarray(mv["images"], dtype=np.float32)
        self.images = imgs
        N, H, W = imgs.shape
        self.N, self.H, self.W = N, H, W
        self.P = attrs["shapePadded"]
        self.sC = zo.shape_cropped(attrs["fouCrop"])
        self.mS = attrs["maxShift"]
        tri = zo.tri_indices(N, attrs["triMode"], attrs.get("diagWidth", 5), 0)
        M = int(tri.sum())
        padded, self.mask = zo.pad_stack(imgs[:2], self.P)
        self.padded = padded
        self.GM, self.MP = zo.mask_spectrum(self.mask, self.sC, self.dt)
        self.nc2 = zo.norm_const2(self.sC)
        self.mmask = zo.max_shift_mask(self.mS)
        self.spec = [zo.frame_spectra(padded[i], self.mask, self.sC, self.dt) for i in range(2)]
        fm = attrs.get("filterMode") or ""
        hot = "hot" in fm
        # a trajectory to shift by, and pair measurements of it to solve
        drift = mv.get("drift")
        self.trans = -(drift - drift.mean(axis=0)) if drift is not None else np.zeros((N, 2))
        units = []

        def registration(tag, n, m, stack, solve=True):
            if hot:
                units.append((tag, "hot", stack))
            units.extend((tag, "spectra", i) for i in range(n))
            units.extend((tag, "pair", i) for i in range(m))
            if solve:
                units.append((tag, "solve", n))
            units.extend((tag, "shift", i) for i in range(n))

        registration("movie", N, M, "movie")
        if "dose" in fm:
            units.append(("movie", "dose_setup", 0))
            units.extend(("movie", "dose_frame", j) for j in range(N))
            units.append(("movie", "dose_finish", 0))
        self.stacks = {"movie": imgs}
        if attrs.get("doEvenOddFRC"):
            # the aligned stack, its even and odd frames, and their sums
            aligned = imgs.copy()
            zo.apply_shifts(aligned, self.trans, originMode=None, dt=self.dt)
            n = N // 2
            self.stacks["even"] = np.ascontiguousarray(aligned[0::2])
            self.stacks["odd"] = np.ascontiguousarray(aligned[1::2])
            self.stacks["sums"] = np.stack([self.stacks["even"].sum(axis=0), self.stacks["odd"].sum(axis=0)])
            registration("even", n, n * (n - 1) // 2, "even")
            registration("odd", N - n, (N - n) * (N - n - 1) // 2, "odd")
            registration("first", 2, 1, "sums", solve=False)
            units.append(("first", "frc", 0))
        else:
            units.append(("movie", "frc", 0))
        self.units = units
        # the movie's filter starts from the default settings; the half sets
        # and the pair of sums get the movie's fitted ones, as the pipeline
        # hands them on (set up here, untimed)
        self.hotinfo = {"movie": dict(zo.DEFAULTS["hotpixInfo"])}
        if hot and len(self.stacks) > 1:
            _, info, _ = zo.hotpix_filter(imgs, dict(zo.DEFAULTS["hotpixInfo"]), dt=self.dt)
            fitted = dict(zo.DEFAULTS["hotpixInfo"])
            fitted.update(info)
            for k in ("even", "odd", "sums"):
                self.hotinfo[k] = fitted
        self._dose = None

    def run(self, unit):
        """Execute one unit (its inputs were prepared in __init__)."""
        zo, dt = self.zo, self.dt
        tag, kind, arg = unit
        if kind == "hot":
            zo.hotpix_filter(self.stacks[arg], dict(self.hotinfo[arg]), dt=dt)
        elif kind == "spectra":
            zo.frame_spectra(self.padded[arg % 2], self.mask, self.sC, dt)
        elif kind == "pair":
            Cw, _ = zo.mnxc2(self.spec[0][0], self.spec[0][1], self.spec[1][0], self.spec[1][1], self.GM, self.MP,
                             self.nc2, self.mS, True, dt)
            zo.locate_peak(Cw, self.mmask, self.attrs.get("subPixReg", 16), self.attrs.get("Bmode", "opti"), dt=dt)
        elif kind == "solve":
            n = arg
            rng = np.random.default_rng(n)
            t = self.trans[:n]
            sh = np.zeros((n, n, 2))
            I, J = np.triu_indices(n, 1)
            sh[I, J] = np.round((t[I] - t[J] + rng.normal(0, 0.05, (len(I), 2))) * 16) / 16
            co = np.zeros((n, n))
            co[I, J] = 1.0
            ps = np.zeros((n, n))
            ps[I, J] = rng.uniform(4.0, 30.0, len(I))
            zo.shifts_solver(sh, co, ps, shapeImage=self.P, maxShift=self.mS)
        elif kind == "shift":
            frame = self.images[arg % 2:arg % 2 + 1].copy()
            zo.apply_shifts(frame, self.trans[arg:arg + 1] + 0.3, originMode=None, dt=dt)
        elif kind == "dose_setup":
            self._dose = zo.dose_filter_setup(self.N, self.P, self.attrs["pixelsize"], self.attrs.get("voltage", 300.0),
                                              self.attrs["doseFiltParam"], self.images[0], dt=dt)
        elif kind == "dose_frame":
            if self._dose is None:
                self.run(("movie", "dose_setup", 0))
            zo.dose_filter_add(self._dose, self.images[arg % 2], arg)
        elif kind == "dose_finish":
            if self._dose is None:
                self.run(("movie", "dose_setup", 0))
            zo.dose_filter_finish(self._dose)
        elif kind == "frc":
            if "sums" in self.stacks:
                zo.tiled_frc(self.stacks["sums"][0], self.stacks["sums"][1], np.vstack([self.trans, self.trans]),
                             dt=dt)
            else:
                zo.lazy_frc(self.images, self.trans, dt=dt)
        else:
            raise ValueError(kind)

    def time_units(self, units):
        out = []
        for u in units:
            t0 = time.perf_counter()
            self.run(u)
            out.append((u, time.perf_counter() - t0))
        return out

    def sample_units(self):
        """The stratified sample: every STRIDE-th unit of each stratum."""
        seen = {}
        out = []
        for u in self.units:
            key = self.stratum(u)
            k = seen.get(key, 0)
            seen[key] = k + 1
            if k % self.STRIDE.get(u[1], 1) == 0:
                out.append(u)
        return out

    def estimate(self, timed):
        """Seconds per movie from timed units: per stratum, the mean unit time
        times the number of units in it."""
        count, tsum, nsmp = {}, {}, {}
        for u in self.units:
            key = self.stratum(u)
            count[key] = count.get(key, 0) + 1
        for u, t in timed:
            key = self.stratum(u)
            tsum[key] = tsum.get(key, 0.0) + t
            nsmp[key] = nsmp.get(key, 0) + 1
        missing = [k for k in count if k not in nsmp]
        if missing:
            raise ValueError("no timed unit of %s" % missing)
        return sum(tsum[k] / nsmp[k] * count[k] for k in count)

    def describe(self):
        kinds = {}
        for u in self.units:
            kinds[u[1]] = kinds.get(u[1], 0) + 1
        return ", ".join("%d %s" % (v, k) for k, v in kinds.items())


def cpu_baseline_sample(mv, attrs, workers):
    """The GPU arm's CPU baseline: the stratified sample of one movie's host
    work, timed, scaled to the movie (seconds per movie, the sample's
    description)."""
    work = HostMovieWork(mv, attrs, workers)
    smp = work.sample_units()
    timed = work.time_units(smp)
    est = work.estimate(timed)
    sampled_s = sum(t for _, t in timed)
    desc = ("stratified sample of one movie's %d host units (%s): every %s-th unit of each stratum (a kind of "
            "unit in the movie, in the two half sets, or in the pair of half sums), %d units timed (%.1f s), "
            "scaled per stratum to the movie" % (
                len(work.units), work.describe(), "/".join("%s %d" % kv for kv in work.STRIDE.items()), len(smp),
                sampled_s))
    return est, desc


def oracle_accuracy(name, mv, reg):
    """Errors of one GPU registration of the workload's seeded movie against
    the float64 oracle's outputs for it (tests/golden/oracle_<name>.npz, made
    by tests/golden/make_bench_oracle.py): drift trajectory RMSE and maximum,
    the half-set trajectories, FRC, and the aligned and dose-filtered sums
    on the fixture's pixel subset.  Empty when there is no fixture or the
    movie differs from the one it was made from."""
    path = os.path.join(ROOT, "tests", "golden", "oracle_%s.npz" % name)
    if not os.path.exists(path):
        return {}
    import hashlib
    g = dict(np.load(path))
    if hashlib.sha256(np.ascontiguousarray(mv["images"], dtype=np.float32).tobytes()).hexdigest() != str(g["checksum"]):
        return {"vs_fp64_oracle": "fixture made from a different movie: not compared"}

    def host(a):
        return a.detach().cpu().numpy() if hasattr(a, "detach") else np.asarray(a)
    tr = host(reg.translations)
    out = {"rmse_vs_fp64_oracle_px": round(float(np.sqrt(np.mean((tr - g["translations"]) ** 2))), 6),
           "max_vs_fp64_oracle_px": round(float(np.abs(tr - g["translations"]).max()), 6),
           "vs_fp64_oracle": "float64 oracle outputs of this seeded movie (tests/golden/oracle_%s.npz)" % name}
    if "transEven" in g and getattr(reg, "transEven", None) is not None:
        out["half_sets_max_vs_fp64_oracle_px"] = round(float(max(np.abs(host(reg.transEven) - g["transEven"]).max(),
                                                               np.abs(host(reg.transOdd) - g["transOdd"]).max())), 6)
    if "FRC" in g and getattr(reg, "FRC", None) is not None:
        out["frc_max_abs_vs_fp64_oracle"] = float("%.3g" % np.nanmax(np.abs(host(reg.FRC) - g["FRC"])))
    for k in ("imageSum", "filtSum"):
        if k + "_idx" in g and getattr(reg, k, None) is not None:
            v = host(getattr(reg, k)).astype(np.float64).reshape(-1)[g[k + "_idx"]]
            out[k + "_rel_l2_vs_fp64_oracle"] = float("%.3g" % (np.linalg.norm(v - g[k + "_val"]) /
                                                              np.linalg.norm(g[k + "_val"])))
    return out


def run_reference(args, wl, rank, world):
    """The reference arm: the reference's algorithm (the float32 CPU
    restatement) on all host cores.  Every unit of one movie's host work is
    timed exactly once over the timed steps: step k runs units k, k + K,
    k + 2K, ... of the movie's unit list (K = --steps), so the K steps
    together are one whole movie, measured; the warm-up steps run slices of
    the same list untimed."""
    if rank != 0:
        return
    from zorro_gb300.synthetic import make_movie
    mv = make_movie(**wl["movie"])
    workers = os.cpu_count() or 1
    work = HostMovieWork(mv, wl["attrs"], workers)
    K = max(1, args.steps)
    slices = [work.units[k::K] for k in range(K)]
    for i in range(args.warmup):
        work.time_units(slices[i % K])
    timed = []
    step_s = []
    for k in range(K):
        t0 = time.perf_counter()
        timed.extend(work.time_units(slices[k]))
        step_s.append(time.perf_counter() - t0)
    movie_s = float(sum(step_s))
    # the GPU arm's stratified estimator applied to the same unit times
    smp = set(work.sample_units())
    est = work.estimate([(u, t) for u, t in timed if u in smp])
    v = 1.0 / movie_s
    by_kind = {}
    for u, t in timed:
        by_kind[u[1]] = by_kind.get(u[1], 0.0) + t
    sample = ("one whole movie measured: all %d host units (%s), unit k of the list in step k mod %d; float32 "
              "restatement of the reference's algorithm, scipy.fft on %d threads for pyFFTW, NumPy for numexprz" % (
                  len(work.units), work.describe(), K, workers))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * movie_s / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded K2-size movie)",
            "config": workload_config(args.workload, args.gpus),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": workers, "kind": "port", "sample": sample,
                             "full_movie_s": round(movie_s, 2), "sampled_estimate_s": round(est, 2),
                             "estimate_vs_full": round(est / movie_s, 3),
                             "seconds_by_kind": {k: round(t, 2) for k, t in by_kind.items()}},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ----------------------------------------------------------------------------- GPU arm

def mixed_sources(torch, dev):
    """The three detector shapes of the batched and served workloads
    (zorro_gb300.workloads.CONFIG4), one seeded 60-frame movie each on the
    device; a movie of n frames is the first n frames of its shape's."""
    from zorro_gb300.workloads import config4_movies
    out = {}
    for name, (mv, attrs, count) in config4_movies(n_frames=60).items():
        raw = torch.from_numpy(mv["raw"]).to(dev)
        gain = torch.from_numpy(mv["gain"]).to(dev) if mv["gain"] is not None else None
        out[name] = (raw, gain, attrs, count, str(mv["raw"].dtype))
    return out


def _mixed_reg(raw, gain, attrs, dev):
    from zorro_gb300.registrator import ImageRegistrator
    r = ImageRegistrator()
    for k, v in attrs.items():
        setattr(r, k, v)
    r.images = raw
    r.gainRef = gain
    r.keepAlignedImages = False
    r.returnDeviceArrays = True
    r.device = dev.index or 0
    return r


def batch_leg(args, torch, dev, lib, dist, world, barrier, sources):
    """The batched uneven workload (CONFIG4): 16 movies, 8 K2 (40 frames),
    5 float16 4096^2 (30 frames), 3 super-resolution (50 frames), each slot
    its own device copy of its shape's movie (the copies' work is real,
    their results equal).  Movies/s of alignImageStacks over the 16 against
    the same 16 through alignImageStack one at a time, and the kernel
    launches of each."""
    from zorro_gb300.registrator import alignImageStacks
    from zorro_gb300.workloads import CONFIG4
    slots = []
    for name, (raw, gain, attrs, count, _) in sources.items():
        n = CONFIG4[name]["movie"]["n_frames"]
        for _ in range(count):
            slots.append((raw[:n].clone(), gain, attrs, name))

    def regs():
        return [_mixed_reg(raw, gain, attrs, dev) for raw, gain, attrs, _ in slots]
    alignImageStacks(regs())
    barrier()
    nb = max(1, min(args.steps, 3))
    l0 = lib.zr_launch_count()
    b0 = torch.cuda.Event(enable_timing=True)
    b1 = torch.cuda.Event(enable_timing=True)
    b0.record()
    for _ in range(nb):
        alignImageStacks(regs())
    b1.record()
    barrier()
    t_batch = slowest_rank(b0.elapsed_time(b1) / 1000.0 / nb, dist, dev)
    launches_batch = (lib.zr_launch_count() - l0) // nb
    # the same movies one at a time (after one warm-up movie of each shape)
    seen = set()
    for r, (_, _, _, name) in zip(regs(), slots):
        if name not in seen:
            seen.add(name)
            r.alignImageStack()
    barrier()
    l0 = lib.zr_launch_count()
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    p0.record()
    for r in regs():
        r.alignImageStack()
    p1.record()
    barrier()
    t_plain = slowest_rank(p0.elapsed_time(p1) / 1000.0, dist, dev)
    launches_plain = lib.zr_launch_count() - l0
    n = len(slots)
    del slots
    return {"value": round(world * n / t_batch, 3), "unit": UNIT, "movies": n,
            "mix": {k: v[3] for k, v in sources.items()},
            "frames": {k: CONFIG4[k]["movie"]["n_frames"] for k in sources},
            "shapes": {k: "%dx%d %s" % (v[0].shape[1], v[0].shape[2], v[4]) for k, v in sources.items()},
            "ms_per_batch": round(t_batch * 1e3, 2), "plain_value": round(world * n / t_plain, 3),
            "vs_plain": round(t_plain / t_batch, 3), "launches_per_batch": int(launches_batch),
            "launches_plain": int(launches_plain)}


def served_mix_leg(args, torch, dev, sources, rank):
    """The served workload (CONFIG5): at each arrival rate, Poisson arrivals
    for ``--poisson-seconds`` seconds, each request a movie of a shape drawn
    50/30/20 with its frame count uniform in [20, 60], admitted by free
    device memory under the 160 GB budget into the server's slots; latency is
    arrival to result.  Per rate: requests, movies/s, p50 and p99."""
    from zorro_gb300.serve import MovieServer
    from zorro_gb300.workloads import CONFIG5
    rng = np.random.default_rng(11 + rank)
    names = list(CONFIG5["mix"])
    probs = np.array([CONFIG5["mix"][k] for k in names])
    lo, hi = CONFIG5["frames"]
    srv = MovieServer(device=dev.index or 0, slots=args.slots, hbm_budget=CONFIG5["hbm_budget"])
    # warm-up: one movie of each shape at the largest frame count
    for name in names:
        raw, gain, attrs, _, _ = sources[name]
        srv.submit(_mixed_reg(raw[:hi], gain, attrs, dev)).result()
    out = []
    for rate in CONFIG5["rates"]:
        srv.reset_stats()
        n_req = max(4, int(round(args.poisson_seconds * rate)))
        gaps = rng.exponential(1.0 / rate, size=n_req)
        picks = rng.choice(len(names), size=n_req, p=probs)
        frames = rng.integers(lo, hi + 1, size=n_req)
        t_next = time.perf_counter()
        futs = []
        for g, k, n in zip(gaps, picks, frames):
            t_next += g
            while time.perf_counter() < t_next:
                time.sleep(min(0.002, max(0.0, t_next - time.perf_counter())))
            raw, gain, attrs, _, _ = sources[names[k]]
            futs.append(srv.submit(_mixed_reg(raw[:int(n)], gain, attrs, dev)))
        for f in futs:
            f.result()
        st_ = srv.stats()
        out.append({"rate_per_s": rate, "requests": n_req,
                    "shapes": {nm: int(np.sum(picks == i)) for i, nm in enumerate(names)},
                    "movies_per_s": round(st_["movies_per_s"], 3), "p50_ms": round(st_["p50_s"] * 1e3, 2),
                    "p99_ms": round(st_["p99_s"] * 1e3, 2)})
    srv.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="k2", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--slots", type=int, default=2, help="movies in flight on the served path")
    ap.add_argument("--profile-only", action="store_true", help="run the warm-up and 2 steps, no timing output")
    ap.add_argument("--no-poisson", action="store_true", help="skip the open-loop Poisson-arrival serving runs")
    ap.add_argument("--poisson-seconds", type=float, default=6.0, help="arrival window per Poisson rate")
    ap.add_argument("--no-fp16", action="store_true", help="skip the half-precision-spectra run")
    ap.add_argument("--no-packed4", action="store_true", help="skip the 4-bit (MRC mode 101) end-to-end run")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched uneven 16-movie run")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, wl, rank, world)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from zorro_gb300.build import build
    if rank == 0:
        build()
    if dist is not None:
        dist.barrier()
    from zorro_gb300 import _lib
    from zorro_gb300.engine import Engine
    from zorro_gb300.registrator import ImageRegistrator
    from zorro_gb300.synthetic import make_movie

    mv = make_movie(**dict(wl["movie"], seed=wl["movie"]["seed"] + rank))
    raw_np = mv["raw"]
    gain_np = mv["gain"]
    b_in = raw_np.dtype.itemsize
    N, H, W = raw_np.shape
    dev = torch.device("cuda", local)
    raw_dev = torch.from_numpy(raw_np).to(dev)
    gain_dev = torch.from_numpy(gain_np).to(dev) if gain_np is not None else None
    raw_pin = torch.from_numpy(raw_np).pin_memory()
    gain_pin = torch.from_numpy(gain_np).pin_memory() if gain_np is not None else None

    def make_reg(images, gain, device_out):
        r = ImageRegistrator()
        for k, v in wl["attrs"].items():
            setattr(r, k, v)
        r.images = images
        r.gainRef = gain
        r.keepAlignedImages = False
        r.returnDeviceArrays = device_out
        r.device = local
        return r

    eng = Engine.get(local)
    lib = _lib.load()
    for _ in range(args.warmup):
        make_reg(raw_dev, gain_dev, True).alignImageStack()
    torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-resident timing (value), with per-stage events
    eng.profile = {}
    launches0 = lib.zr_launch_count()
    barrier()
    with ClockSampler(local) as clk:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        ev0.record()
        last = None
        for _ in range(args.steps):
            last = make_reg(raw_dev, gain_dev, True)
            last.alignImageStack()
        ev1.record()
        barrier()
        wall = time.perf_counter() - t0
    launches = lib.zr_launch_count() - launches0
    dev_ms = ev0.elapsed_time(ev1)
    stage_ms = eng.stage_ms()
    host_ms = eng.host_ms()
    eng.profile = None
    if args.profile_only:
        return
    t_step = max(dev_ms / 1000.0, 1e-9) / args.steps
    t_step = slowest_rank(t_step, dist, dev)
    value = world / t_step

    # ---- the same movies with half-precision frame spectra (spectraPrecision 'float16')
    fp16 = None
    Cc = int(wl["attrs"]["fouCrop"][0])
    if not args.no_fp16:
        def make_reg16():
            r = make_reg(raw_dev, gain_dev, True)
            r.spectraPrecision = "float16"
            return r
        for _ in range(2):
            make_reg16().alignImageStack()
        barrier()
        h0 = torch.cuda.Event(enable_timing=True)
        h1 = torch.cuda.Event(enable_timing=True)
        h0.record()
        last16 = None
        for _ in range(args.steps):
            last16 = make_reg16()
            last16.alignImageStack()
        h1.record()
        barrier()
        t16 = slowest_rank(h0.elapsed_time(h1) / 1000.0 / args.steps, dist, dev)
        fp16 = {"value": round(world / t16, 3), "unit": UNIT, "ms_per_step": round(t16 * 1e3, 3),
                "spectra_bytes_half": int(2 * N * (Cc // 2 + 1) * Cc * 4),
                "spectra_bytes_float": int(2 * N * (Cc // 2 + 1) * Cc * 8)}
        if rank == 0:
            # the half-precision movie against the float64 oracle's outputs
            fp16["accuracy"] = {k: v for k, v in oracle_accuracy(args.workload, mv, last16).items()
                                if k != "vs_fp64_oracle"}

    # ---- served path: movies in flight in parallel slots (continuous batching)
    from zorro_gb300.serve import MovieServer
    srv = MovieServer(device=local, slots=args.slots, hbm_budget=160e9)
    for _ in range(args.slots):
        srv.submit(make_reg(raw_dev, gain_dev, True)).result()
    srv.reset_stats()
    barrier()
    sv0 = time.perf_counter()
    futs = [srv.submit(make_reg(raw_dev, gain_dev, True)) for _ in range(args.steps * args.slots)]
    for f in futs:
        f.result()
    barrier()
    t_served = (time.perf_counter() - sv0) / (args.steps * args.slots)
    served = srv.stats()
    srv.close()
    t_served = slowest_rank(t_served, dist, dev)

    # ---- end to end through the public API from pinned host memory, after
    # warm-up steps of its own (the first host-input movie allocates its
    # device copy of the frames and the pinned output buffers)
    for _ in range(max(args.warmup, 1)):
        make_reg(raw_pin, gain_pin, False).alignImageStack()
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        r = make_reg(raw_pin, gain_pin, False)
        r.alignImageStack()
        _ = (r.translations, r.imageSum, r.filtSum, r.FRC)
    e1.record()
    barrier()
    t_e2e = e0.elapsed_time(e1) / 1000.0 / args.steps
    t_e2e = slowest_rank(t_e2e, dist, dev)
    h2d = raw_np.nbytes + (gain_np.nbytes if gain_np is not None else 0)
    d2h = 4 * H * W * 2 + 512 * 512 * 4 + 256 * 8 + N * 2 * 8

    # ---- end to end from a packed 4-bit movie (the MRC mode-101 layout of
    # counting detectors: the same counts clipped to 15, two pixels a byte);
    # the packed bytes cross the host link and zr_unpack_u4 expands them
    packed4 = None
    if not args.no_packed4 and raw_np.dtype == np.uint8:
        from zorro_gb300.mrc import Packed4
        c4 = np.minimum(raw_np, 15)
        if W % 2:
            c4 = np.concatenate([c4, np.zeros((N, H, 1), np.uint8)], axis=2)
        pk = torch.from_numpy(np.ascontiguousarray(c4[..., 0::2] | (c4[..., 1::2] << 4))).pin_memory()
        p4 = Packed4(pk.numpy(), (N, H, W))
        for _ in range(2):
            make_reg(p4, gain_pin, False).alignImageStack()
        barrier()
        q0 = torch.cuda.Event(enable_timing=True)
        q1 = torch.cuda.Event(enable_timing=True)
        q0.record()
        for _ in range(args.steps):
            r = make_reg(p4, gain_pin, False)
            r.alignImageStack()
            _ = (r.translations, r.imageSum, r.filtSum, r.FRC)
        q1.record()
        barrier()
        t4 = slowest_rank(q0.elapsed_time(q1) / 1000.0 / args.steps, dist, dev)
        # the unpack kernel alone: packed bytes read + uint8 frames written
        pk_dev = pk.to(dev).reshape(-1)
        u8_dev = torch.empty((N, H, W), dtype=torch.uint8, device=dev)
        st_ = torch.cuda.current_stream(dev).cuda_stream
        for _ in range(3):
            lib.zr_unpack_u4(ctypes.c_void_p(pk_dev.data_ptr()), N, H, W, ctypes.c_void_p(u8_dev.data_ptr()),
                             ctypes.c_void_p(st_))
        u0 = torch.cuda.Event(enable_timing=True)
        u1 = torch.cuda.Event(enable_timing=True)
        u0.record()
        for _ in range(10):
            lib.zr_unpack_u4(ctypes.c_void_p(pk_dev.data_ptr()), N, H, W, ctypes.c_void_p(u8_dev.data_ptr()),
                             ctypes.c_void_p(st_))
        u1.record()
        torch.cuda.synchronize()
        t_unpack = u0.elapsed_time(u1) / 10.0 / 1000.0
        peak_, _ = measured_peaks()
        ub = pk.numel() + N * H * W
        packed4 = {"value": round(world / t4, 3), "unit": UNIT,
                   "h2d_bytes_per_step": int(pk.numel() + (gain_np.nbytes if gain_np is not None else 0)),
                   "d2h_bytes_per_step": d2h, "input": "the K2 counts clipped to 15, packed 4-bit (MRC mode 101)",
                   "unpack_ms": round(t_unpack * 1e3, 4), "unpack_gbs": round(ub / t_unpack / 1e9, 1),
                   "unpack_frac": round(ub / t_unpack / 1e9 / peak_, 3)}

    # ---- batched uneven launch: 16 movies of three detector shapes (8 K2,
    # 5 float16 4096^2, 3 super-resolution binned 2x) registered as one batch,
    # against the same 16 movies registered one at a time
    batched = served_mix = None
    if not (args.no_batch and args.no_poisson):
        sources = mixed_sources(torch, dev)
        if not args.no_batch:
            batched = batch_leg(args, torch, dev, lib, dist, world, barrier, sources)
        if not args.no_poisson:
            served_mix = served_mix_leg(args, torch, dev, sources, rank)
        del sources

    # ---- roofline of the dominant stage
    w = 2 * wl["attrs"]["maxShift"]
    C = int(wl["attrs"]["fouCrop"][0])
    M = N * (N - 1) // 2 if wl["attrs"]["triMode"] == "tri" else None
    evenodd = bool(wl["attrs"].get("doEvenOddFRC"))
    ab = algorithmic_bytes(N, H, W, C, w, M, b_in, evenodd=evenodd, hot="hot" in wl["attrs"].get("filterMode", ""))
    per_step = {k: v / args.steps for k, v in stage_ms.items()}
    dom = max(per_step, key=per_step.get)
    peak, peak_kind = measured_peaks()
    achieved = ab[dom] / (per_step[dom] / 1000.0) / 1e9
    traffic = read_traffic().get(dom) if args.workload == "k2" else None
    P = int(wl["attrs"]["shapePadded"][0])
    fl = fft_flops(N, P, C, w, M if M is not None else N - 1, evenodd=evenodd)
    # FP32 CUDA-core peak: 152 SMs x 128 lanes x 2 FLOP x SM clock
    fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12
    roof = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "peak_kind": peak_kind,
            "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
            "traffic_gbs": round(traffic / (per_step[dom] / 1000.0) / 1e9, 1) if traffic else None,
            "algorithmic_bytes": ab[dom], "stage_ms_per_step": {k: round(v, 3) for k, v in sorted(per_step.items())},
            "movie_algorithmic_bytes": sum(ab.values()),
            "movie_frac": round(sum(ab.values()) / t_step / 1e9 / peak, 4),
            "fft_tflops": {k: round(v / (per_step[k] / 1000.0) / 1e12, 2) for k, v in fl.items() if k in per_step},
            "fp32_peak_tflops": round(fp32_peak, 1),
            "host_ms_per_step": {k: round(v / args.steps, 3) for k, v in sorted(host_ms.items())}}

    # ---- where one movie's time goes: device busy and idle, host steps
    timeline = movie_timeline(eng, torch, lambda: make_reg(raw_dev, gain_dev, True).alignImageStack())

    # ---- accuracy of the last timed movie (outside the timed region): against
    # the known drift, and against the float64 oracle's outputs for this
    # seeded movie (tests/golden/oracle_<workload>.npz)
    tr = np.asarray(last.translations)
    truth = -(mv["drift"] - mv["drift"].mean(axis=0))
    accuracy = {"rmse_vs_true_drift_px": round(float(np.sqrt(np.mean((tr - truth) ** 2))), 4)}
    if rank == 0:
        accuracy.update(oracle_accuracy(args.workload, mv, last))

    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline and world == 1:
            workers = os.cpu_count() or 1
            s, sample = cpu_baseline_sample(mv, wl["attrs"], workers)
            cpu = {"value": 1.0 / s, "unit": UNIT, "cores": workers, "kind": "port", "sample": sample,
                   "sampled_estimate_s": round(s, 2)}
        line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(t_step * 1000.0, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded K2-size movies)",
                "config": workload_config(args.workload, world),
                "e2e": {"value": round(world / t_e2e, 3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "served": {"value": round(world / t_served, 3), "unit": UNIT, "slots": args.slots,
                           "p50_ms": round(served["p50_s"] * 1e3, 2), "p99_ms": round(served["p99_s"] * 1e3, 2),
                           "vs_plain": round((world / t_served) / value, 3)},
                "served_mix": served_mix,
                "fp16_spectra": fp16,
                "e2e_packed4": packed4,
                "batched": batched,
                "gpu_launches": int(launches),
                "wall_s_timed": round(wall, 3),
                "clocks": clk.summary(),
                "roofline": roof,
                "timeline": timeline,
                "accuracy": accuracy,
                "cpu_baseline": cpu}
        if not args.profile_only:
            print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

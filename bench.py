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

``--impl reference`` times the reference algorithm on the host cores: the
float32 CPU restatement of the same pipeline (NumPy/SciPy, FFTs on all
cores), on a bounded sample of each movie, scaled to a whole movie.
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

K2_DOSE = [1.2 * 1.05 ** 2, 0.24499, -1.6649, 2.8141, 32, 0]
WORKLOADS = {
    "k2": dict(movie=dict(n_frames=40, shape=(3838, 3710), seed=2024, mean_dose=0.8, drift_sigma=1.2, dtype="uint8",
                          gain_map=True, hot_fraction=1e-4, hot_factor=50.0),
               attrs=dict(triMode="tri", shapePadded=[4096, 4096], fouCrop=[2048, 2048], maxShift=100,
                          pixelsize=0.105, voltage=300.0, filterMode="hot,dose", doseFiltParam=K2_DOSE,
                          subPixReg=16, shiftMethod="lanczos", Bmode="opti", doEvenOddFRC=True)),
    # the K2 movie cut to 10 frames (142 MB of raw frames, still larger than L2): the case the
    # per-kernel ncu captures run on
    "k2x10": dict(movie=dict(n_frames=10, shape=(3838, 3710), seed=2024, mean_dose=0.8, drift_sigma=1.2,
                             dtype="uint8", gain_map=True, hot_fraction=1e-4, hot_factor=50.0),
                  attrs=dict(triMode="tri", shapePadded=[4096, 4096], fouCrop=[2048, 2048], maxShift=100,
                             pixelsize=0.105, voltage=300.0, filterMode="hot,dose", doseFiltParam=K2_DOSE,
                             subPixReg=16, shiftMethod="lanczos", Bmode="opti", doEvenOddFRC=True)),
    "small": dict(movie=dict(n_frames=20, shape=(1024, 1024), seed=1, mean_dose=1.0, drift_sigma=0.8),
                  attrs=dict(triMode="tri", shapePadded=[1024, 1024], fouCrop=[1024, 1024], maxShift=40,
                             pixelsize=0.1, voltage=300.0, filterMode="dose",
                             doseFiltParam=[1.0, 0.24499, -1.6649, 2.8141, 32, 0], subPixReg=16)),
}
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

def cpu_sample(mv, attrs, workers, pairs=2, frames=1, full_steps=False):
    """Time the float32 CPU restatement (the reference's algorithm) on a
    bounded sample of one movie and scale it to the whole movie.

    Sample: the hot-pixel filter on the whole stack once (when full_steps),
    the forward spectra of ``frames`` frames, ``pairs`` pair correlations with
    their peak search, and the shift, FRC-sum and dose-filter work of
    ``frames`` frames.  Per-movie time = hot + N*spectra + M*pair + N*(shift +
    dose) + solve."""
    from oracle import zorro_oracle as zo
    dt = zo.Dtypes(False, workers)
    N, H, W = mv["images"].shape
    P = attrs["shapePadded"]
    sC = zo.shape_cropped(attrs["fouCrop"])
    mS = attrs["maxShift"]
    tri = zo.tri_indices(N, attrs["triMode"], attrs.get("diagWidth", 5), 0)
    M = int(tri.sum())
    imgs = mv["images"][:max(frames, 2)].astype(np.float32)
    t = {}
    t0 = time.perf_counter()
    if full_steps and "hot" in (attrs.get("filterMode") or ""):
        zo.hotpix_filter(mv["images"], dict(zo.DEFAULTS["hotpixInfo"]), dt=dt)
    t["hot"] = time.perf_counter() - t0
    padded, mask = zo.pad_stack(imgs, P)
    t0 = time.perf_counter()
    GM, MP = zo.mask_spectrum(mask, sC, dt)
    spec = [zo.frame_spectra(padded[i], mask, sC, dt) for i in range(max(frames, 2))]
    t["spectra_per_frame"] = (time.perf_counter() - t0) / max(frames, 2)
    nc2 = zo.norm_const2(sC)
    mmask = zo.max_shift_mask(mS)
    t0 = time.perf_counter()
    for _ in range(pairs):
        Cw, _ = zo.mnxc2(spec[0][0], spec[0][1], spec[1][0], spec[1][1], GM, MP, nc2, mS, True, dt)
        zo.locate_peak(Cw, mmask, attrs.get("subPixReg", 16), "opti", dt=dt)
    t["pair"] = (time.perf_counter() - t0) / pairs
    trans = np.zeros((frames, 2)) + 0.3
    t0 = time.perf_counter()
    zo.apply_shifts(imgs[:frames].copy(), trans, originMode=None)
    t["shift_per_frame"] = (time.perf_counter() - t0) / frames
    t0 = time.perf_counter()
    if "dose" in (attrs.get("filterMode") or ""):
        zo.dose_filter(imgs[:frames], P, attrs["pixelsize"], 300.0, attrs["doseFiltParam"],
                       np.zeros((H, W), np.float32), dt=dt)
    t["dose_per_frame"] = (time.perf_counter() - t0) / frames
    per_frame = t["spectra_per_frame"] + t["shift_per_frame"] + t["dose_per_frame"]
    movie_s = t["hot"] + N * per_frame + M * t["pair"]
    extra = ""
    if attrs.get("doEvenOddFRC"):
        # evenOddFouRingCorr (zorro.py:2099-2224): the even and the odd frames
        # registered again with the saved settings (hot filter, spectra, the
        # half triangle, shifts, dose), then the two sums in 'first' mode
        n = N // 2
        Mh = n * (n - 1) // 2
        movie_s += 2 * (t["hot"] * n / N + n * per_frame + Mh * t["pair"]) + 2 * t["spectra_per_frame"] + t["pair"]
        extra = " + two half-set registrations of %d frames / %d pairs and the 'first' pair of the sums" % (n, Mh)
    return movie_s, t, "hot-pixel filter of the full stack %s, spectra of %d frames, %d of %d pairs, shift and dose " \
        "of %d frame(s); scaled to %d frames / %d pairs%s" % ("(timed)" if full_steps else "(not in sample)",
                                                               max(frames, 2), pairs, M, frames, N, M, extra)


def run_reference(args, wl, rank, world):
    if rank != 0:
        return
    from zorro_gb300.synthetic import make_movie
    mv = make_movie(**wl["movie"])
    workers = os.cpu_count() or 1
    vals = []
    sample = ""
    for i in range(args.warmup + args.steps):
        s, _, sample = cpu_sample(mv, wl["attrs"], workers, pairs=1, frames=1, full_steps=(i == 0))
        if i == 0:
            hot_s = _
        if i >= args.warmup:
            vals.append(1.0 / (s + hot_s.get("hot", 0.0)))
    v = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded K2-size movie)",
            "config": workload_config(args.workload, args.gpus),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": workers, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ----------------------------------------------------------------------------- GPU arm

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
    ap.add_argument("--poisson-seconds", type=float, default=3.0, help="arrival window per Poisson rate")
    ap.add_argument("--no-fp16", action="store_true", help="skip the half-precision-spectra run")
    ap.add_argument("--no-packed4", action="store_true", help="skip the 4-bit (MRC mode 101) end-to-end run")
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
        for _ in range(args.steps):
            make_reg16().alignImageStack()
        h1.record()
        barrier()
        t16 = slowest_rank(h0.elapsed_time(h1) / 1000.0 / args.steps, dist, dev)
        fp16 = {"value": round(world / t16, 3), "unit": UNIT, "ms_per_step": round(t16 * 1e3, 3),
                "spectra_bytes_half": int(2 * N * (Cc // 2 + 1) * Cc * 4),
                "spectra_bytes_float": int(2 * N * (Cc // 2 + 1) * Cc * 8)}

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
    # open-loop serving: Poisson arrivals at fixed rates, latency = arrival to result
    poisson = []
    if not args.no_poisson:
        rng = np.random.default_rng(7 + rank)
        for rate in (2.0, 8.0, 32.0):
            srv.reset_stats()
            n_req = max(8, int(args.poisson_seconds * rate))
            gaps = rng.exponential(1.0 / rate, size=n_req)
            t_start = time.perf_counter()
            futs = []
            for g in gaps:
                t_start += g
                while time.perf_counter() < t_start:
                    time.sleep(min(0.002, max(0.0, t_start - time.perf_counter())))
                futs.append(srv.submit(make_reg(raw_dev, gain_dev, True)))
            for f in futs:
                f.result()
            st_ = srv.stats()
            poisson.append({"rate_per_s": rate, "requests": n_req, "movies_per_s": round(st_["movies_per_s"], 3),
                            "p50_ms": round(st_["p50_s"] * 1e3, 2), "p99_ms": round(st_["p99_s"] * 1e3, 2)})
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
            "fp32_peak_tflops": round(fp32_peak, 1)}

    # ---- accuracy on this movie vs the known drift (the float64 oracle comparison is in the tests)
    tr = np.asarray(last.translations)
    truth = -(mv["drift"] - mv["drift"].mean(axis=0))
    rmse_truth = float(np.sqrt(np.mean((tr - truth) ** 2)))

    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline and world == 1:
            workers = os.cpu_count() or 1
            s, parts, sample = cpu_sample(mv, wl["attrs"], workers, pairs=3, frames=1, full_steps=True)
            cpu = {"value": 1.0 / s, "unit": UNIT, "cores": workers, "kind": "port", "sample": sample,
                   "seconds_per_movie": round(s, 2)}
        line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(t_step * 1000.0, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded K2-size movies)",
                "config": workload_config(args.workload, world),
                "e2e": {"value": round(world / t_e2e, 3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "served": {"value": round(world / t_served, 3), "unit": UNIT, "slots": args.slots,
                           "p50_ms": round(served["p50_s"] * 1e3, 2), "p99_ms": round(served["p99_s"] * 1e3, 2),
                           "vs_plain": round((world / t_served) / value, 3), "poisson": poisson},
                "fp16_spectra": fp16,
                "e2e_packed4": packed4,
                "gpu_launches": int(launches),
                "wall_s_timed": round(wall, 3),
                "clocks": clk.summary(),
                "roofline": roof,
                "accuracy": {"rmse_vs_true_drift_px": round(rmse_truth, 4)},
                "cpu_baseline": cpu}
        if not args.profile_only:
            print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

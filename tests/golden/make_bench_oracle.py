"""Float64 oracle outputs of the benchmark's K2 movie (and other named
workloads), for the GPU parity test at the full benchmark size and for the
benchmark's accuracy figure.

    python tests/golden/make_bench_oracle.py [--out DIR] [workload ...]     (default: k2)

Each workload's seeded synthetic movie (``zorro_gb300.workloads``) goes
through ``oracle.zorro_oracle.align_image_stack`` in float64 with FFTs on all
host cores; ``tests/golden/oracle_<workload>.npz`` stores the input checksum,
the drift trajectories (movie and even/odd half sets), the pair matrices,
the FRC, the hot-pixel counts and a fixed subset of the aligned and
dose-filtered sums with their totals.  The oracle is itself pinned against
the unmodified reference by the fixtures of ``make_golden.py``.

The K2 fixture is made on the aarch64 host of the GB300 machines, where the
benchmark and the GPU tests run: the seeded K2 movie is 570 million Poisson
draws, and the few-ulp differences between the x86 and aarch64 builds of
NumPy/SciPy (FFT and exp) change a handful of them, so a fixture made on one
platform does not match the movie generated on the other (the input checksum
says which).
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from tests.golden.make_golden import input_checksum, subset  # noqa: E402
from zorro_gb300.synthetic import make_movie  # noqa: E402
from zorro_gb300.workloads import workload  # noqa: E402


def fixture_path(name, out_dir=None):
    return os.path.join(out_dir or os.path.join(ROOT, "tests", "golden"), "oracle_%s.npz" % name)


def main(names, out_dir=None):
    from oracle import zorro_oracle as zo
    for name in names:
        mk, attrs = workload(name)
        mv = make_movie(**mk)
        t0 = time.time()
        ref = zo.align_image_stack(mv["images"], workers=os.cpu_count(), **attrs)
        ed = ref["errorDict"]
        out = {"checksum": np.array(input_checksum(mv["images"])), "oracle_seconds": np.array(time.time() - t0)}
        for k in ("shiftsTriMat", "corrTriMat", "peaksigTriMat"):
            out[k] = np.asarray(ed[k], dtype=np.float64)
        out["translations"] = np.asarray(ref["translations"], dtype=np.float64)
        for k in ("transEven", "transOdd", "FRC"):
            if k in ref:
                out[k] = np.asarray(ref[k], dtype=np.float64)
        subset("imageSum", ref["imageSum"], out)
        if "filtSum" in ref:
            subset("filtSum", ref["filtSum"], out)
        if "hotpixInfo" in ref:
            for k in ("guessDeadpix", "guessHotpix", "neighborPix"):
                out["hot_" + k] = np.array(ref["hotpixInfo"][k])
        path = fixture_path(name, out_dir)
        np.savez_compressed(path, **out)
        print("wrote %s (%d bytes, oracle %.0f s)" % (path, os.path.getsize(path), float(out["oracle_seconds"])))


if __name__ == "__main__":
    args = sys.argv[1:]
    out_dir = None
    if args[:1] == ["--out"]:
        out_dir, args = args[1], args[2:]
    main(args or ["k2"], out_dir)

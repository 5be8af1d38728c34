"""The directory watcher on the GPU: movies dropped into a directory are
registered through a MovieServer (two slots) and their sums equal the
API's; a movie the GPU path refuses ends as a zombie with its error, the
others complete."""
import os
import threading
import time

import numpy as np
import pytest

from oracle import mrc_oracle as mo
from zorro_gb300 import watch
from zorro_gb300.registrator import ImageRegistrator
from zorro_gb300.serve import MovieServer
from zorro_gb300.synthetic import make_movie

pytestmark = pytest.mark.gpu
ATTRS = dict(triMode="tri", shapePadded=[256, 256], fouCrop=[128, 128], maxShift=20)


def test_watcher_registers_dropped_movies(tmp_path):
    inp, out = tmp_path / "in", tmp_path / "out"
    inp.mkdir()
    movies = {}
    for i, seed in enumerate((3, 4)):
        mv = make_movie(10, (200, 180), seed=seed, mean_dose=2.0, drift_sigma=0.8, dtype="uint8")
        movies["m%d" % i] = mv["raw"]
        mo.write(str(inp / ("m%d.mrc" % i)), mv["raw"], 0, pixelsize_nm=0.1)
    mo.write(str(inp / "big.mrc"), np.zeros((3, 40, 5000), np.uint8), 0)  # wider than the padded size
    default = ImageRegistrator()
    for k, v in ATTRS.items():
        setattr(default, k, v)
    default.saveMovie = False
    srv = MovieServer(slots=2)
    w = watch.MovieWatcher(str(inp), default=default, output_dir=str(out), server=srv, min_size=1, wait_time=0.0)
    stop = threading.Event()
    th = threading.Thread(target=w.run, args=(stop, 0.05))
    th.start()
    t0 = time.time()
    while (not w.jobs or w.busy()) and time.time() - t0 < 120:
        time.sleep(0.1)
    stop.set()
    th.join()
    srv.close()
    st = w.statuses()
    assert st == {"m0.mrc": "complete", "m1.mrc": "complete", "big.mrc": "zombie"}, (st, w.errors())
    assert "shapePadded" in w.errors()["big.mrc"]
    for name, raw in movies.items():
        s, _, _ = mo.read(str(out / "sum" / ("%s_zorro.mrc" % name)))
        api = ImageRegistrator()
        for k, v in ATTRS.items():
            setattr(api, k, v)
        api.images = raw
        api.alignImageStack()
        assert np.array_equal(s[0], api.imageSum)
        cfg = ImageRegistrator()
        cfg.loadConfig(str(out / (name + ".zor")))
        assert cfg.METAstatus == "fini" and np.array_equal(cfg.translations, api.translations)

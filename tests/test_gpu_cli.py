"""The command line end to end on the GPU (zorro/__main__.py: loadConfig with
loadData, alignImageStack, saveData, saveConfig): the sums and trajectory it
writes equal an in-process registration of the same movie."""
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import mrc_oracle as mo
from zorro_gb300.registrator import ImageRegistrator
from zorro_gb300.synthetic import make_movie

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ATTRS = dict(triMode="tri", shapePadded=[256, 256], fouCrop=[128, 128], maxShift=20, filterMode="dose",
             doseFiltParam=[1.0, 0.24499, -1.6649, 2.8141, 32, 0])


@pytest.mark.parametrize("use_i", [False, True])
def test_cli_registers_like_the_api(tmp_path, use_i):
    mv = make_movie(12, (200, 180), seed=4, mean_dose=2.0, drift_sigma=0.8, dtype="uint8")
    mo.write(str(tmp_path / "movie.mrc"), mv["raw"], 0, pixelsize_nm=0.1)
    cfg = ImageRegistrator()
    for k, v in ATTRS.items():
        setattr(cfg, k, v)
    cfg.files["stack"] = "movie.mrc"
    cfg.saveConfig(str(tmp_path / "movie.zor"))
    args = [sys.executable, "-m", "zorro_gb300", "-c", "movie.zor", "-o", "out/sum.mrc"]
    if use_i:
        args += ["-i", "movie.mrc"]
    r = subprocess.run(args, cwd=tmp_path, capture_output=True, text=True, env=dict(os.environ, PYTHONPATH=ROOT))
    assert r.returncode == 0, r.stdout + r.stderr
    done = ImageRegistrator()
    done.loadConfig(str(tmp_path / "movie.zor"))
    assert done.METAstatus == "fini"
    s, _, ps = mo.read(str(tmp_path / "out" / "sum.mrc"))
    f, _, _ = mo.read(str(tmp_path / "out" / "sum_filt.mrc"))
    api = ImageRegistrator()
    for k, v in ATTRS.items():
        setattr(api, k, v)
    api.images = mv["raw"]
    api.pixelsize = np.float32(0.1)
    api.alignImageStack()
    assert np.array_equal(done.translations, api.translations)
    assert np.array_equal(s[0], api.imageSum) and np.array_equal(f[0], api.filtSum)
    assert abs(ps - 0.1) < 1e-6

"""The .zor configs (ImageRegistrator.saveConfig / loadConfig,
zorro/zorro.py:3682-4075) and the command line (zorro/__main__.py) against
the reference's own outputs: tests/golden/config_ref.zor was written by the
unmodified reference's saveConfig and config_ref_loaded.json records what its
loadConfig set from that file (tests/golden/make_config_golden.py)."""
import json
import os
import subprocess
import sys

import numpy as np

from tests.golden.make_config_golden import LOADED_ATTRS, config_state, to_json
from zorro_gb300 import __main__ as cli
from zorro_gb300.registrator import ImageRegistrator

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def configured():
    reg = ImageRegistrator()
    for k, v in config_state().items():
        setattr(reg, k, v)
    return reg


def test_save_config_matches_reference_file(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    reg = configured()
    reg.saveConfig("config_ref.zor")
    with open(os.path.join(GOLDEN, "config_ref.zor")) as fh:
        want = fh.read()
    assert open("config_ref.zor").read() == want


def test_load_config_matches_reference(tmp_path, monkeypatch):
    with open(os.path.join(GOLDEN, "config_ref_loaded.json")) as fh:
        want = json.load(fh)
    monkeypatch.chdir(GOLDEN)
    reg = ImageRegistrator()
    reg.loadConfig("config_ref.zor")
    for k in LOADED_ATTRS:
        assert to_json(getattr(reg, k, "<unset>")) == want[k], k
    # the reference's reading quirks
    assert reg.doFRC is False and reg.doLazyFRC is True   # doLazyFRC is read into doFRC
    assert reg.ctfInfo["AmplitudeContrast"] == 0.07        # CTFInfo is read into ctfInfo
    assert reg.errorDictList[0]["single"] == 4.0 and reg.errorDictList[0]["M"] == 3


def test_round_trip_and_loaded_data(tmp_path, monkeypatch):
    from oracle import mrc_oracle as mo
    monkeypatch.chdir(tmp_path)
    raw = np.random.default_rng(1).integers(0, 8, size=(3, 8, 10)).astype(np.uint8)
    mo.write("m.mrc", raw, 0, pixelsize_nm=0.2)
    a = configured()
    a.files["stack"] = "m.mrc"
    a.files["gainRef"] = None
    a.saveConfig("a.zor")
    b = ImageRegistrator()
    b.loadConfig("a.zor", loadData=True)
    assert np.array_equal(b.images, raw) and b.pixelsize == np.float32(0.2)
    for k in ("triMode", "fouCrop", "maxShift", "filterMode", "doseFiltParam", "hotpixInfo", "gainInfo"):
        assert to_json(getattr(b, k)) == to_json(getattr(a, k) if k != "fouCrop" else np.array(a.fouCrop)), k
    assert np.array_equal(b.translations, a.translations)


def test_missing_config_raises(tmp_path):
    import pytest
    with pytest.raises(IOError):
        ImageRegistrator().loadConfig(str(tmp_path / "nope.zor"))


def test_cli_template_and_arguments(tmp_path):
    r = subprocess.run([sys.executable, "-m", "zorro_gb300"], cwd=tmp_path, capture_output=True, text=True,
                       env=dict(os.environ, PYTHONPATH=ROOT))
    assert r.returncode == 0, r.stderr
    t = ImageRegistrator()
    t.loadConfig(str(tmp_path / "template.zor"))
    assert t.triMode == "diag" and t.maxShift == 100 and list(t.fouCrop) == [3072, 3072]
    assert cli.parse(["-c", "x.zor", "-i", "m.mrc", "-o", "s.mrc"]) == ("x.zor", "m.mrc", "s.mrc")
    assert cli.parse(["-i", "m.mrc"]) == (None, "m.mrc", None)

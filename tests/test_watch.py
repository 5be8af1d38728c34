"""The directory watcher's state machine (the reference's Skulk states,
automator/zorroSkulkManager.py:243-350), on the CPU: a fake clock and file
stats drive it, and a fake server stands in for the GPU slots."""
import concurrent.futures as cf
import os
import types

import numpy as np

from oracle import mrc_oracle as mo
from zorro_gb300 import watch
from zorro_gb300.registrator import ImageRegistrator


class FakeFS:
    def __init__(self):
        self.files = {}

    def stat(self, name):
        if name not in self.files:
            raise FileNotFoundError(name)
        size, mtime = self.files[name]
        return types.SimpleNamespace(st_size=size, st_mtime=mtime)


class FakeServer:
    """Resolves every request at once; ``fail`` names movies whose registration raises."""

    def __init__(self, fail=()):
        self.order, self.fail = [], set(fail)

    def submit(self, reg):
        self.order.append(os.path.basename(reg.files["stack"]))
        f = cf.Future()
        if os.path.basename(reg.files["stack"]) in self.fail:
            f.set_exception(ValueError("kernel refused the movie"))
        else:
            reg.imageSum = np.zeros((4, 4), np.float32)
            reg.translations = np.zeros((3, 2))
            f.set_result(reg)
        return f


def _watcher(tmp_path, fs, server, clock):
    d = ImageRegistrator()
    d.saveMovie = False
    return watch.MovieWatcher(str(tmp_path), default=d, server=server, min_size=100, wait_time=5.0,
                              clock=lambda: clock[0], stat=fs.stat)


def _touch(tmp_path, name, nz=3):
    p = str(tmp_path / name)
    mo.write(p, np.zeros((nz, 4, 4), np.uint8), 0)
    return p


def test_stability_rule_and_completion(tmp_path):
    fs, srv, clock = FakeFS(), FakeServer(), [0.0]
    w = _watcher(tmp_path, fs, srv, clock)
    p = _touch(tmp_path, "a.mrc")
    fs.files[p] = (50, 1.0)                        # still being written, small
    w.poll(); assert w.statuses()["a.mrc"] == "changing"
    fs.files[p] = (200, 2.0)                       # grew: the wait restarts
    clock[0] = 1; w.poll(); assert w.statuses()["a.mrc"] == "changing"
    clock[0] = 2; w.poll()                         # unchanged: the wait starts now
    clock[0] = 6; w.poll(); assert w.statuses()["a.mrc"] == "changing"   # 4 s < 5 s
    clock[0] = 8; w.poll(); assert w.statuses()["a.mrc"] == "stable"
    assert w.poll() == 1                           # ready -> submitted -> done
    assert w.statuses()["a.mrc"] == "complete" and not w.busy()
    done = ImageRegistrator()
    done.loadConfig(str(tmp_path / "a.zor"))
    assert done.METAstatus == "fini" and os.path.isfile(str(tmp_path / "sum" / "a_zorro.mrc"))


def test_small_files_never_stable(tmp_path):
    fs, srv, clock = FakeFS(), FakeServer(), [0.0]
    w = _watcher(tmp_path, fs, srv, clock)
    p = _touch(tmp_path, "tiny.mrc")
    fs.files[p] = (99, 1.0)
    for t in range(0, 60, 5):
        clock[0] = t
        w.poll()
    assert w.statuses()["tiny.mrc"] == "changing" and srv.order == []


def test_newest_movie_first(tmp_path):
    fs, srv, clock = FakeFS(), FakeServer(), [0.0]
    w = _watcher(tmp_path, fs, srv, clock)
    for name, mt in (("old.mrc", 10.0), ("new.mrc", 20.0), ("mid.mrc", 15.0)):
        fs.files[_touch(tmp_path, name)] = (500, mt)
    for t in (0, 1, 2, 10, 11, 12):
        clock[0] = t
        w.poll()
    assert srv.order == ["new.mrc", "mid.mrc", "old.mrc"]


def test_errors_become_statuses(tmp_path):
    fs, srv, clock = FakeFS(), FakeServer(fail={"bad.mrc"}), [0.0]
    w = _watcher(tmp_path, fs, srv, clock)
    fs.files[_touch(tmp_path, "bad.mrc")] = (500, 1.0)
    fs.files[_touch(tmp_path, "good.mrc")] = (500, 2.0)
    junk = str(tmp_path / "junk.mrc")
    open(junk, "wb").write(b"not an mrc file" * 100)
    fs.files[junk] = (1500, 3.0)
    for t in (0, 1, 2, 10, 11, 12, 13):
        clock[0] = t
        w.poll()
    st = w.statuses()
    assert st["good.mrc"] == "complete"
    assert st["bad.mrc"] == "zombie" and st["junk.mrc"] == "zombie"
    assert "kernel refused" in w.errors()["bad.mrc"]
    cfg = ImageRegistrator()
    cfg.loadConfig(str(tmp_path / "bad.zor"))
    assert cfg.METAstatus == "error"


def test_config_files_are_ready_at_once(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)  # the config's relative output names resolve here
    fs, srv, clock = FakeFS(), FakeServer(), [0.0]
    w = _watcher(tmp_path, fs, srv, clock)
    movie = _touch(tmp_path, "m.mrc")
    job_dir = tmp_path / "jobs"
    job_dir.mkdir()
    r = ImageRegistrator()
    r.files["stack"] = movie
    r.saveMovie = False
    r.saveConfig(str(job_dir / "m.zor"))
    w2 = watch.MovieWatcher(str(job_dir), server=srv, clock=lambda: clock[0], stat=fs.stat)
    fs.files[str(job_dir / "m.zor")] = (10, 1.0)
    w2.poll()
    assert w2.statuses()["m.zor"] == "changing"
    w2.poll()
    assert w2.statuses()["m.zor"] == "complete" and srv.order == ["m.mrc"]
    assert os.path.isfile(str(tmp_path / "sum" / "m_zorro.mrc"))

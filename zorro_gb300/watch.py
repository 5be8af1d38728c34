"""Directory watcher feeding the GPU request loop: the registration side of
the reference's Skulk daemon (automator/zorroSkulkManager.py:69-350).

A ``MovieWatcher`` polls an input directory.  Every new movie (``*.mrc``,
``*.mrcs``) or config (``*.zor``) becomes a job that walks the reference's
states:

    new -> changing -> stable -> ready -> proc -> fini -> complete
                                      \\-> error -> zombie

* changing -> stable: a movie is stable once two consecutive polls see the
  same size and modification time, the size is at least ``min_size``
  (1 MiB, as the reference's __MIN_FILE_SIZE), and a further ``wait_time``
  (5 s) has passed without change, because acquisition software writes
  slowly (zorroSkulkManager.py:259-289); a .zor config is ready at once;
* stable: the job's priority is the movie's modification time, so the newest
  movie is registered first (zorroSkulkManager.py:232-237, 292-296);
* ready: the job's registrator is the default config (a .zor or an
  ``ImageRegistrator``) with the reference's file names for this movie;
  its config is written with METAstatus 'ready' and the movie is read;
* proc: ``alignImageStack`` runs in a slot of a ``MovieServer`` (several
  movies in flight on one GPU, admission by device memory);
* fini/complete: the sums are saved (``saveData``) and the config written
  back with METAstatus 'fini';
* error/zombie: any exception of a job (an unreadable movie, a size the
  GPU path does not take, a failed kernel) is kept as the job's status and
  written to its config with METAstatus 'error'; the other jobs go on.

Files are not moved or compressed (the reference's renaming into its raw
directory and its archiving step are not part of the registration path).
``clock`` and ``stat`` can be replaced (tests drive the state machine
without waiting).
"""
from __future__ import annotations

import copy
import glob
import os
import threading
import time

NEW, CHANGING, STABLE, READY, PROCESSING, FINISHED, COMPLETE, ERROR, ZOMBIE = range(9)
STATE_NAMES = {NEW: "new", CHANGING: "changing", STABLE: "stable", READY: "ready", PROCESSING: "proc",
               FINISHED: "fini", COMPLETE: "complete", ERROR: "error", ZOMBIE: "zombie"}
MOVIE_EXTS = (".mrc", ".mrcs")
CONFIG_EXTS = (".zor",)


class Job:
    """One watched file and its registration."""

    def __init__(self, name):
        self.name = name
        self.state = NEW
        self.priority = -1.0
        self.prior_mtime = None
        self.prior_size = None
        self.wait = -1.0
        self.reg = None
        self.future = None
        self.error = None

    @property
    def statename(self):
        return STATE_NAMES[self.state]


class MovieWatcher:
    """Register the movies that appear in ``input_dir``.

    ``default``: a .zor path or an ``ImageRegistrator`` whose settings every
    movie gets; ``output_dir``: where configs and sums go (default: the
    input directory); ``server``: a ``MovieServer`` (made on first use when
    None), or any object with ``submit(reg) -> Future``."""

    def __init__(self, input_dir, default=None, output_dir=None, server=None, min_size=1 << 20, wait_time=5.0,
                 clock=time.time, stat=os.stat):
        self.input_dir = os.path.abspath(input_dir)
        self.output_dir = os.path.abspath(output_dir or input_dir)
        self.default = default
        self.server = server
        self.min_size = int(min_size)
        self.wait_time = float(wait_time)
        self.clock = clock
        self.stat = stat
        self.jobs = {}
        self._lock = threading.Lock()

    # ------------------------------------------------------------------ jobs
    def _template(self):
        from .registrator import ImageRegistrator
        if isinstance(self.default, str):
            reg = ImageRegistrator()
            reg.loadConfig(self.default)
            reg.files["config"] = None
            reg.files["stack"] = None
            return reg
        return copy.deepcopy(self.default) if self.default is not None else ImageRegistrator()

    def _make_registrator(self, job):
        """The job's registrator with the reference's default names for its
        movie (sum/<movie>_zorro.mrc, align/<movie>_zorro_movie.mrcs and
        <movie>.zor under the output directory)."""
        from .registrator import ImageRegistrator
        if job.name.endswith(CONFIG_EXTS):
            reg = ImageRegistrator()
            reg.loadConfig(job.name)
            return reg
        reg = self._template()
        front = os.path.splitext(os.path.basename(job.name))[0]
        reg.files = dict(reg.files)
        reg.files["stack"] = job.name
        reg.files["config"] = os.path.join(self.output_dir, front + ".zor")
        reg.files["sum"] = os.path.join(self.output_dir, "sum", "%s_zorro.mrc" % front)
        reg.files["align"] = os.path.join(self.output_dir, "align", "%s_zorro_movie.mrcs" % front)
        reg.files["filt"] = None
        return reg

    def _fail(self, job, exc):
        job.error = "%s: %s" % (type(exc).__name__, exc)
        job.state = ERROR
        if job.reg is not None:
            job.reg.METAstatus = "error"
            try:
                job.reg.saveConfig()
            except Exception:
                pass

    def _finish(self, job):
        try:
            job.future.result()
            job.state = FINISHED
            job.reg.saveData()
            job.reg.METAstatus = "fini"
            job.reg.saveConfig()
            job.state = COMPLETE
            job.priority = -1.0
        except Exception as exc:  # noqa: BLE001 - every failure becomes the job's status
            self._fail(job, exc)

    def _submit(self, job):
        if self.server is None:
            from .serve import MovieServer
            self.server = MovieServer()
        try:
            job.reg = self._make_registrator(job)
            job.reg.METAstatus = "ready"
            job.reg.saveConfig()
            job.reg.loadData()
            job.state = PROCESSING
            job.reg.METAstatus = "proc"
            job.future = self.server.submit(job.reg)
            job.future.add_done_callback(lambda _f, j=job: self._finish(j))
        except Exception as exc:  # noqa: BLE001
            self._fail(job, exc)

    # ------------------------------------------------------------------ polling
    def _update(self, job):
        """One step of the job's state machine (zorroSkulkManager.py:243-350)."""
        if job.state == NEW:
            st = self.stat(job.name)
            job.prior_mtime, job.prior_size = st.st_mtime, st.st_size
            job.state = CHANGING
        elif job.state == CHANGING:
            if job.name.endswith(CONFIG_EXTS):
                job.state = READY
                return
            st = self.stat(job.name)
            if st.st_mtime == job.prior_mtime and st.st_size == job.prior_size and st.st_size >= self.min_size:
                if job.wait < 0.0:
                    job.wait = self.clock()
                elif job.wait + self.wait_time < self.clock():
                    job.state = STABLE
            else:
                job.wait = -1.0
            job.prior_mtime, job.prior_size = st.st_mtime, st.st_size
        elif job.state == STABLE:
            job.priority = self.stat(job.name).st_mtime
            job.state = READY
        elif job.state == ERROR:
            job.state = ZOMBIE
            job.priority = -1e6

    def poll(self):
        """One cycle: pick up new files, advance every job, submit the ready
        ones (newest movie first).  Returns the number of jobs submitted."""
        names = []
        for ext in MOVIE_EXTS + CONFIG_EXTS:
            names += glob.glob(os.path.join(self.input_dir, "*" + ext))
        with self._lock:
            for n in sorted(names):
                if n not in self.jobs:
                    self.jobs[n] = Job(n)
            for job in list(self.jobs.values()):
                try:
                    self._update(job)
                except OSError as exc:  # the file went away
                    self._fail(job, exc)
            ready = sorted((j for j in self.jobs.values() if j.state == READY), key=lambda j: -j.priority)
        for job in ready:
            self._submit(job)
        return len(ready)

    def statuses(self):
        with self._lock:
            return {os.path.basename(n): j.statename for n, j in self.jobs.items()}

    def errors(self):
        with self._lock:
            return {os.path.basename(n): j.error for n, j in self.jobs.items() if j.error}

    def busy(self):
        with self._lock:
            return any(j.state not in (COMPLETE, ZOMBIE) for j in self.jobs.values())

    def run(self, stop, interval=1.0):
        """Poll every ``interval`` seconds until ``stop`` (a threading.Event) is set."""
        while not stop.is_set():
            self.poll()
            stop.wait(interval)

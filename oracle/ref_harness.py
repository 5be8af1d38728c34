"""Run the UNMODIFIED Zorro reference pipeline in float64 on the CPU.

TEST INFRASTRUCTURE ONLY.  This module loads ``zorro/zorro.py`` and
``zorro/zorro_util.py`` from a read-only checkout of LBEM-CH/zorro and runs
``ImageRegistrator.alignImageStack`` on seeded synthetic movies.  It exists to
produce golden fixtures (``tests/golden/``) that pin the numpy restatement in
``oracle/zorro_oracle.py``.  It only works where that checkout exists; nothing
on the product path, in the GPU tests or in ``bench.py`` imports it.

What the harness supplies, because the reference's runtime dependencies are
absent or unbuildable here:

* stub modules ``matplotlib``, ``mpl_toolkits...anchored_artists``, ``mrcz``
  and ``zorro_plotting`` (plotting and file I/O only);
* ``pyfftw.builders.fft2/ifft2`` stand-ins on ``scipy.fft`` with the
  ``update_arrays``/``execute`` protocol the reference uses
  (``zorro_util.py:1041,1047``).  The reference always runs its plans with
  ``FFTW.execute()``, which applies no scaling in either direction (pyFFTW
  applies ``normalise_idft`` only in ``FFTW.__call__``); the reference's own
  factors (``normConst2`` in mnxc2, ``normConst`` in applyShifts and
  binStack) are written for those unscaled inverses, so the stand-in's
  inverse is unscaled too (``norm="forward"``);
* a ``numexprz.evaluate`` stand-in that evaluates the expression string with
  NumPy on the caller's frame (the reference's 60 ``nz.evaluate`` sites);
* ``np.int``/``np.float``/``np.Inf`` aliases removed in NumPy 2;
* in-memory source edits for NumPy-2 compatibility (listed in
  ``_COMPAT_EDITS``; one restores NumPy < 1.14's ``lstsq`` error on an empty
  system, which ``hotpixFilter`` relies on to fall back to its default
  cut-offs, ``zorro.py:2572-2592``) plus the fix for the ``missingDose`` UnboundLocalError in
  ``doseFilter`` (``zorro.py:2408-2417``) when ``doseFiltParam[0]`` is set;
* a deterministic shift solve: the reference minimises the weighted L1 norm
  ``sum(w*|A x - b|)`` (``zorro_util.py:849-851``) with the stochastic
  ``scipy.optimize.basinhopping`` (``zorro.py:1415,1422``).  Here that call is
  answered by the exact optimum of the same objective (linear programme,
  HiGHS).  The logistic fit's basinhopping (``zorro.py:2008``) is answered by
  the deterministic Nelder-Mead minimisation of the same objective from the
  same start point within the same bounds
  (``oracle.zorro_oracle.logistic_fit_deterministic``) (basinhopping is
  chaotic here: 1e-9 changes of its input change the fit by O(1)).

The float dtypes are switched to float64/complex128 after loading, the way
the reference itself selects them when numexprz is absent (``zorro.py:20-29``).
"""
from __future__ import annotations

import contextlib
import io
import os
import sys
import tempfile
import types
import warnings

import numpy as np
import scipy.fft
import scipy.optimize

# The checkout of LBEM-CH/zorro to run: required, no default (the harness
# runs only where a reference checkout exists; nothing on the GPU path does).
REF_ROOT = os.environ.get("ZORRO_REF_ROOT")


def ref_root():
    """The reference checkout named by ZORRO_REF_ROOT (its zorro/zorro.py must exist)."""
    if not REF_ROOT:
        raise RuntimeError("set ZORRO_REF_ROOT to a checkout of LBEM-CH/zorro (the directory holding zorro/zorro.py)")
    if not os.path.exists(os.path.join(REF_ROOT, "zorro", "zorro.py")):
        raise RuntimeError("ZORRO_REF_ROOT=%s holds no zorro/zorro.py" % REF_ROOT)
    return REF_ROOT

# (line number, old text, new text) -- applied to the source text before
# compiling, so reported line numbers stay those of the reference file.
_COMPAT_EDITS = [
    (584, "self.masks == []", "len(self.masks) == 0"),
    (1301, "np.argwhere(triIndices[I,:])[-1] + 1", "np.argwhere(triIndices[I,:])[-1][0] + 1"),
    (1990, "if bins == None:", "if bins is None:"),
    (2452, "qvect[ np.argwhere( np.abs(doseFinish - optiDoseVect) < np.abs(doseStart - optiDoseVect) )[-1] ]",
     "qvect[ np.argwhere( np.abs(doseFinish - optiDoseVect) < np.abs(doseStart - optiDoseVect) )[-1][0] ]"),
    # missingDose is only defined when doseFiltParam[0] is None (zorro.py:2408-2413)
    # NumPy < 1.14 raised LinAlgError from lstsq on an empty system, which sent
    # hotpixFilter to its default cut-offs; NumPy 2 returns zeros (-> NaN)
    (2576, "np.linalg.lstsq(", "_lstsq_strict("),
    (2587, "np.linalg.lstsq(", "_lstsq_strict("),
    (2413, "dosePerFrame = self.doseFiltParam[0]",
     "dosePerFrame = self.doseFiltParam[0]; missingDose = dosePerFrame * np.float32( self.doseFiltParam[5] )"),
    # evenOddFouRingCorr's sub-registrators load the parent's config, including
    # doEvenOddFRC=True, and recurse until a half-set has too few frames for
    # cdfLogisticCurve (zorro.py:2128-2186): one level only
    (2128, "evenReg.loadConfig( tempLogName )", "evenReg.loadConfig( tempLogName ); evenReg.doEvenOddFRC = False"),
    (2132, "oddReg.loadConfig( tempLogName )", "oddReg.loadConfig( tempLogName ); oddReg.doEvenOddFRC = False"),
    (2186, "eoReg.loadConfig( tempLogName )", "eoReg.loadConfig( tempLogName ); eoReg.doEvenOddFRC = False"),
]

_NE_FUNCS = {
    "real": np.real, "imag": np.imag, "conj": np.conj, "abs": np.abs,
    "sqrt": np.sqrt, "exp": np.exp, "log": np.log, "sin": np.sin, "cos": np.cos,
    "arctan2": np.arctan2, "where": np.where,
}

def _lstsq_strict(a, b, *args, **kw):
    """``np.linalg.lstsq`` as NumPy < 1.14 behaved: empty systems raise."""
    a = np.asarray(a)
    if a.size == 0:
        raise np.linalg.LinAlgError("Arrays cannot be empty")
    return np.linalg.lstsq(a, b, rcond=None)


def _ne_evaluate(ex, local_dict=None, global_dict=None, out=None, **_kw):
    frame = sys._getframe(1)
    ns = dict(frame.f_globals)
    ns.update(frame.f_locals if local_dict is None else local_dict)
    ns.update(_NE_FUNCS)
    with np.errstate(all="ignore"):
        val = eval(ex, {"__builtins__": {}}, ns)
    val = np.asarray(val)
    if out is not None:
        out[...] = val
        return out
    return val


class _Plan:
    def __init__(self, inverse, workers):
        self.inverse = inverse
        self.workers = workers
        self.i = self.o = None

    def update_arrays(self, i, o):
        self.i, self.o = i, o

    def execute(self):
        # FFTW.execute(): the plain transform, no 1/N on the inverse
        if self.inverse:
            self.o[...] = scipy.fft.ifft2(self.i, norm="forward", workers=self.workers)
        else:
            self.o[...] = scipy.fft.fft2(self.i, workers=self.workers)


def _make_stubs(workers):
    mods = {}
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    plt.__getattr__ = lambda name: (lambda *a, **k: None)
    mpl.pyplot = plt
    mpl.use = lambda *a, **k: None
    mods["matplotlib"] = mpl
    mods["matplotlib.pyplot"] = plt
    tk = types.ModuleType("mpl_toolkits")
    ag = types.ModuleType("mpl_toolkits.axes_grid1")
    aa = types.ModuleType("mpl_toolkits.axes_grid1.anchored_artists")
    tk.axes_grid1 = ag
    ag.anchored_artists = aa
    mods["mpl_toolkits"] = tk
    mods["mpl_toolkits.axes_grid1"] = ag
    mods["mpl_toolkits.axes_grid1.anchored_artists"] = aa
    mrcz = types.ModuleType("mrcz")
    mrcz.writeMRC = lambda *a, **k: None
    mrcz.readMRC = lambda *a, **k: (_ for _ in ()).throw(IOError("mrcz stub"))
    mods["mrcz"] = mrcz
    zp = types.ModuleType("zorro_plotting")
    zp.generate = lambda *a, **k: None
    mods["zorro_plotting"] = zp
    pf = types.ModuleType("pyfftw")
    bl = types.ModuleType("pyfftw.builders")
    bl.fft2 = lambda a, **k: _Plan(False, workers)
    bl.ifft2 = lambda a, **k: _Plan(True, workers)
    pf.builders = bl
    pf.import_wisdom = lambda *a, **k: None
    pf.export_wisdom = lambda *a, **k: ()
    mods["pyfftw"] = pf
    mods["pyfftw.builders"] = bl
    ne = types.ModuleType("numexprz")
    ne.evaluate = _ne_evaluate
    ne.nthreads = workers
    ne.set_num_threads = lambda n: None
    ne.detect_number_of_cores = lambda: workers
    mods["numexprz"] = ne
    return mods


class _SolverShim:
    """Stands in for ``scipy.optimize`` inside the loaded reference module.

    ``basinhopping`` on the reference's shift objective is answered with the
    exact weighted-L1 optimum; on the logistic objective by a deterministic
    minimisation (both from ``oracle.zorro_oracle``)."""

    def __init__(self, util):
        self._util = util

    def __getattr__(self, name):
        return getattr(scipy.optimize, name)

    def basinhopping(self, func, x0, niter=100, minimizer_kwargs=None, **kw):
        mk = dict(minimizer_kwargs or {})
        if func is self._util.weightedErrorNorm:
            A, b, w = mk["args"]
            bounds = mk["bounds"]
            from oracle.zorro_oracle import weighted_l1_exact
            return types.SimpleNamespace(x=weighted_l1_exact(A, b, w, bounds))
        if func is self._util.minLogistic:
            from oracle.zorro_oracle import logistic_fit_deterministic
            hSigma, cdf = mk["args"]
            (lo, hi) = mk["bounds"][0]
            return types.SimpleNamespace(x=logistic_fit_deterministic(hSigma, cdf, lo, hi, x0[0]))
        raise RuntimeError("unexpected basinhopping objective %r" % func)


_LOADED = {}
_STUBS = {}


@contextlib.contextmanager
def _stubs_installed(workers=None):
    """Install the stub modules for the duration of a load or a run (the
    reference imports pyfftw lazily inside ``pyFFTWPlanner``)."""
    if not _STUBS:
        _STUBS.update(_make_stubs(workers or os.cpu_count()))
    saved = {k: sys.modules.get(k) for k in _STUBS}
    sys.modules.update(_STUBS)
    try:
        yield
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v


def load_reference(fp64=True, workers=None):
    """Return the loaded reference ``zorro`` module (cached per dtype)."""
    key = (fp64,)
    if key in _LOADED:
        return _LOADED[key]
    workers = workers or os.cpu_count()
    sys.dont_write_bytecode = True
    for alias, val in (("int", int), ("float", float), ("Inf", np.inf), ("NaN", np.nan)):
        if not hasattr(np, alias):
            setattr(np, alias, val)
    with _stubs_installed(workers), warnings.catch_warnings():
        warnings.simplefilter("ignore")
        util = types.ModuleType("zorro_util")
        upath = os.path.join(ref_root(), "zorro", "zorro_util.py")
        util.__file__ = upath
        with open(upath) as fh:
            exec(compile(fh.read(), upath, "exec"), util.__dict__)
        sys.modules["zorro_util"] = util
        zpath = os.path.join(ref_root(), "zorro", "zorro.py")
        with open(zpath) as fh:
            lines = fh.read().split("\n")
        for lineno, old, new in _COMPAT_EDITS:
            if old not in lines[lineno - 1]:
                raise RuntimeError("compat edit does not match zorro.py:%d" % lineno)
            lines[lineno - 1] = lines[lineno - 1].replace(old, new)
        zmod = types.ModuleType("zorro_ref_fp64" if fp64 else "zorro_ref_fp32")
        zmod.__file__ = zpath
        with contextlib.redirect_stdout(io.StringIO()):
            exec(compile("\n".join(lines), zpath, "exec"), zmod.__dict__)
        zmod._lstsq_strict = _lstsq_strict
        if fp64:
            zmod.fftw_dtype = "complex128"
            zmod.float_dtype = "float64"
        zmod.scipy = types.SimpleNamespace(optimize=_SolverShim(util), ndimage=__import__("scipy.ndimage").ndimage,
                                           stats=__import__("scipy.stats").stats,
                                           special=__import__("scipy.special").special)
        zmod._harness_util = util
        sys.modules.pop("zorro_util", None)
    _LOADED[key] = zmod
    return zmod


def run_reference(images, *, fp64=True, capture=False, **attrs):
    """Run ``alignImageStack`` on ``images`` with the given attributes.

    Returns the registrator.  With ``capture=True`` the per-pair correlation
    windows (``C`` before and after the B-filter), the optimal Gaussian sigma
    and the forward spectra of the first frame are recorded on the object as
    ``_cap``."""
    zmod = load_reference(fp64=fp64)
    reg = zmod.ImageRegistrator()
    reg.verbose = 0
    reg.images = images
    with tempfile.TemporaryDirectory() as td:
        reg.cachePath = td
        for k, v in attrs.items():
            setattr(reg, k, v)
        # evenOddFouRingCorr writes a temporary .zor into the working directory
        # and names its half-set sums after files['sum'] (zorro.py:2121-2215)
        reg.files = dict(reg.files)
        if not reg.files.get("sum"):
            reg.files["sum"] = os.path.join(td, "sum.mrc")
        cap = {"C": {}, "Cfilt": {}, "sigma": {}}
        if capture:
            orig_locate = zmod.ImageRegistrator.locatePeak
            orig_min = zmod.scipy.optimize.__class__

            def locate(self, I, J, _orig=orig_locate):
                cap["C"][(int(I), int(J))] = np.array(self._ImageRegistrator__C)
                _orig(self, I, J)
                cap["Cfilt"][(int(I), int(J))] = np.array(self._ImageRegistrator__C_filt)

            reg.locatePeak = types.MethodType(locate, reg)
        cwd = os.getcwd()
        os.chdir(td)
        try:
            with _stubs_installed(), contextlib.redirect_stdout(io.StringIO()), np.errstate(all="ignore"):
                reg.alignImageStack()
        finally:
            os.chdir(cwd)
        if capture:
            reg._cap = cap
    return reg

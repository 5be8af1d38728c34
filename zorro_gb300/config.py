""".zor configuration files: ``ImageRegistrator.saveConfig`` / ``loadConfig``
(zorro.py:3682-4075).

A .zor file is an INI file (``configparser.RawConfigParser``, keys case
sensitive, comment lines stored as keys without values) with the sections
initialization, calibration, registration, ctf, io, plot, results, data and
one errorDict<n> section per entry of ``errorDictList``.  Lists, dicts and
arrays are JSON; scalars are written with ``str()``.

The layout below is the reference's, entry for entry and in its order, so
that a file written here equals the one the reference writes for the same
state, and each file loads into the same attributes.  The reference's
reading rules are kept with their quirks, because configs written by one
are read by the other:

* every read is optional: a missing or unparsable value leaves the
  attribute as it was;
* ``None`` is written as a key without a value and reads back as ``None``
  for text entries (numbers and flags then keep their previous value);
* ``doLazyFRC`` is read into ``doFRC`` (zorro.py:3860), ``BfiltType`` is
  read under a key the writer spells ``BFiltType`` (zorro.py:3846, 4002; so
  it is never read back), and ``CTFInfo`` is read into ``ctfInfo``
  (zorro.py:3774);
* the integer entries of the writer go through ``int()`` and are left out
  when that fails (``n_threads = None``);
* saved error dictionaries are appended to ``errorDictList``; arrays of one
  element come back as scalars.
"""
from __future__ import annotations

import configparser
import json
import os

import numpy as np

_C = "comment"   # a comment line (a key without a value)
_S = "str"       # str(value)
_I = "int"       # str(int(value)), left out when int() fails
_J = "json"      # json.dumps(value), arrays as lists
_JN = "json_if"  # json, only when the value is not None
_JA = "json_arr"  # json of value.tolist(), only when not None

# (section, key, attribute or comment text, kind), in the writer's order
_LAYOUT = [
    ("initialization", "METAstatus", "METAstatus", _S),
    ("initialization", "# METAstatus _MUST_ appear as second line in file", None, _C),
    ("initialization", "# For detailed use instructions: github.com/C-CINA/zorro/wiki", None, _C),
    ("initialization", "verbose", "verbose", _S),
    ("initialization", "umask", "umask", _S),
    ("initialization", "fftw_effort", "fftw_effort", _S),
    ("initialization", "# n_threads is usually best if set to the number of physical cores (CPUs)", None, _C),
    ("initialization", "n_threads", "n_threads", _I),
    ("initialization", "saveC", "saveC", _S),
    ("initialization", "cachePath", "cachePath", _S),
    ("calibration", "# Zorro can strip this information from .DM4 files if its is present in tags", None, _C),
    ("calibration", "# Pixel size in nanometers", None, _C),
    ("calibration", "pixelsize", "pixelsize", _S),
    ("calibration", "# Accelerating voltage in kV", None, _C),
    ("calibration", "voltage", "voltage", _S),
    ("calibration", "# Spherical aberration in mm", None, _C),
    ("calibration", "C3", "C3", _S),
    ("calibration", "# Gain in electrons/count", None, _C),
    ("calibration", "gain", "gain", _S),
    ("calibration", "detectorPixelSize", "detectorPixelSize", _S),
    ("calibration", "gainInfo", "gainInfo", _J),
    ("registration", "xcorrMode", "xcorrMode", _S),
    ("registration", "# tri, diag, first, auto, or autocorr", None, _C),
    ("registration", "triMode", "triMode", _S),
    ("registration", "# Use a padding 10 % bigger than the original image, select an efficient size with "
                     "zorro_util.findValidFFTWDim()", "shapePadded", _C),
    ("registration", "shapePadded", "shapePadded", _JN),
    ("registration", "shapeOriginal", "shapeOriginal", _JN),
    ("registration", "shapeBinned", "shapeBinned", _JN),
    ("registration", "fouCrop", "fouCrop", _JN),
    ("registration", "subPixReg", "subPixReg", _I),
    ("registration", "shiftMethod", "shiftMethod", _S),
    ("registration", "# Maximum shift in pixels within diagWidth/autoMax frames", None, _C),
    ("registration", "maxShift", "maxShift", _I),
    ("registration", "# preShift = True is useful for crystalline specimens where you want maxShift to follow the "
                     "previous frame position", None, _C),
    ("registration", "preShift", "preShift", _S),
    ("registration", "diagStart", "diagStart", _I),
    ("registration", "diagWidth", "diagWidth", _I),
    ("registration", "autoMax", "autoMax", _I),
    ("registration", "startFrame", "startFrame", _I),
    ("registration", "endFrame", "endFrame", _I),
    ("registration", "# peakSigThres changes with dose but usually is uniform for a dataset", None, _C),
    ("registration", "peaksigThres", "peaksigThres", _S),
    ("registration", "# corrThres is DEPRECATED", None, _C),
    ("registration", "corrThres", "corrThres", _S),
    ("registration", "velocityThres", "velocityThres", _S),
    ("registration", "# Brad is radius of B-filter in Fourier pixels", None, _C),
    ("registration", "Brad", "Brad", _S),
    ("registration", "# Bmode = conv, opti, or fourier", None, _C),
    ("registration", "Bmode", "Bmode", _S),
    ("registration", "BFiltType", "BfiltType", _S),
    ("registration", "# originMode is centroid, or (empty), empty sets frame 1 to (0,0)", None, _C),
    ("registration", "originMode", "originMode", _S),
    ("registration", "# weightMode is one of logistic, corr, norm, unweighted", None, _C),
    ("registration", "weightMode", "weightMode", _S),
    ("registration", "logisticK", "logisticK", _S),
    ("registration", "logisticNu", "logisticNu", _S),
    ("registration", "# Set suppressOrigin = True if gain reference artifacts are excessive", None, _C),
    ("registration", "suppressOrigin", "suppressOrigin", _S),
    ("registration", "filterMode", "filterMode", _S),
    ("registration", "doLazyFRC", "doLazyFRC", _S),
    ("registration", "doEvenOddFRC", "doEvenOddFRC", _S),
    ("registration", "doseFiltParam", "doseFiltParam", "dose"),
    ("ctf", "CTFProgram", "CTFProgram", _S),
    ("ctf", "CTFInfo", "CTFInfo", _J),
    ("io", "savePNG", "savePNG", _S),
    ("io", "compress_ext", "compress_ext", _S),
    ("io", "saveMovie", "saveMovie", _S),
    ("io", "doCompression", "doCompression", _S),
    ("io", "# Note: all paths are relative to the current working directory.", None, _C),
    ("io", "files", "files", _J),
    ("plot", "plotDict", "plotDict", _J),
    ("results", "translations", "translations", _JA),
    ("results", "transEven", "transEven", _JA),
    ("results", "transOdd", "transOdd", _JA),
    ("results", "rotations", "rotations", _JA),
    ("results", "scales", "scales", _JA),
    ("results", "velocities", "velocities", _JA),
    ("results", "FRC", "FRC", _JA),
    ("data", "hotpixInfo", "hotpixInfo", _J),
    ("data", "trackCorrStats", "trackCorrStats", _S),
    ("data", "corrStats", "corrStats", _J),
    ("data", "bench", "bench", _J),
]

# (section, key, attribute, parser) in the reader's order; the attribute
# names differ from the writer's keys where the reference's do
_READS = [
    ("initialization", "verbose", "verbose", "int"), ("initialization", "umask", "umask", "int"),
    ("initialization", "fftw_effort", "fftw_effort", "upper"), ("initialization", "n_threads", "n_threads", "int"),
    ("initialization", "saveC", "saveC", "bool"), ("initialization", "METAstatus", "METAstatus", "str"),
    ("initialization", "cachePath", "cachePath", "str"),
    ("calibration", "pixelsize", "pixelsize", "float"), ("calibration", "voltage", "voltage", "float"),
    ("calibration", "C3", "C3", "float"), ("calibration", "gain", "gain", "float"),
    ("calibration", "detectorPixelSize", "detectorPixelSize", "float"),
    ("calibration", "gainInfo", "gainInfo", "json"),
    ("data", "trackCorrStats", "trackCorrStats", "bool"), ("data", "corrStats", "corrStats", "json"),
    ("data", "bench", "bench", "json"), ("data", "hotpixInfo", "hotpixInfo", "json"),
    ("results", "translations", "translations", "array"), ("results", "transEven", "transEven", "array"),
    ("results", "transOdd", "transOdd", "array"), ("results", "velocities", "velocities", "array"),
    ("results", "rotations", "rotations", "array"), ("results", "scales", "scales", "array"),
    ("results", "FRC", "FRC", "array"),
    ("ctf", "CTFProgram", "CTFProgram", "str"), ("ctf", "CTFInfo", "ctfInfo", "json"),
    "errorDicts",
    ("registration", "xcorrMode", "xcorrMode", "str"), ("registration", "triMode", "triMode", "str"),
    ("registration", "startFrame", "startFrame", "int"), ("registration", "endFrame", "endFrame", "int"),
    ("registration", "shapePadded", "shapePadded", "array"),
    ("registration", "shapeOriginal", "shapeOriginal", "array"),
    ("registration", "shapeBinned", "shapeBinned", "array"), ("registration", "fouCrop", "fouCrop", "array"),
    ("registration", "subPixReg", "subPixReg", "int"), ("registration", "shiftMethod", "shiftMethod", "str"),
    ("registration", "maxShift", "maxShift", "int"), ("registration", "preShift", "preShift", "bool"),
    ("registration", "triMode", "triMode", "str"), ("registration", "diagWidth", "diagWidth", "int"),
    ("registration", "diagStart", "diagStart", "int"), ("registration", "autoMax", "autoMax", "int"),
    ("registration", "peaksigThres", "peaksigThres", "float"),
    ("registration", "corrThres", "corrThres", "float"),
    ("registration", "velocityThres", "velocityThres", "float"), ("registration", "Brad", "Brad", "float"),
    ("registration", "Bmode", "Bmode", "str"), ("registration", "BfiltType", "BfiltType", "str"),
    ("registration", "originMode", "originMode", "str"),
    ("registration", "suppressOrigin", "suppressOrigin", "bool"),
    ("registration", "weightMode", "weightMode", "str"), ("registration", "logisticK", "logisticK", "float"),
    ("registration", "logisticNu", "logisticNu", "float"), ("registration", "filterMode", "filterMode", "str"),
    ("registration", "doLazyFRC", "doFRC", "bool"), ("registration", "doEvenOddFRC", "doEvenOddFRC", "bool"),
    ("registration", "doseFiltParam", "doseFiltParam", "json"),
    ("io", "files", "files", "json"), ("io", "savePNG", "savePNG", "bool"),
    ("io", "compress_ext", "compress_ext", "str"), ("io", "saveMovie", "saveMovie", "bool"),
    ("io", "doCompression", "doCompression", "bool"),
    ("plot", "plotDict", "plotDict", "json"),
]


def _jsonable(v):
    if isinstance(v, np.ndarray):
        return v.tolist()
    if isinstance(v, np.generic):
        return v.item()
    raise TypeError("%r is not JSON serialisable" % (v,))


def _dumps(v):
    return json.dumps(v.tolist() if isinstance(v, np.ndarray) else v, default=_jsonable)


def _parser():
    cp = configparser.RawConfigParser(allow_no_value=True)
    cp.optionxform = str
    return cp


def save_config(reg, configNameIn=None):
    """Write ``reg``'s state as a .zor file (zorro.py:3889-4075); returns the path."""
    if not configNameIn:
        if reg.files.get("config") is None:
            reg.files["config"] = str(reg.files.get("stack")) + ".zor"
    else:
        reg.files["config"] = configNameIn
    path = reg.files["config"]
    d = os.path.realpath(os.path.dirname(path))
    if d and not os.path.isdir(d):
        os.mkdir(d)
    cp = _parser()
    for section, key, attr, kind in _LAYOUT:
        if not cp.has_section(section):
            cp.add_section(section)
        if kind == _C:
            if attr is None or getattr(reg, attr, None) is not None:
                cp.set(section, key)
            continue
        v = getattr(reg, attr, None)
        if kind == _S:
            cp.set(section, key, None if v is None else str(v))  # None: a bare key, read back as None
        elif kind == _I:
            try:
                cp.set(section, key, str(int(v)))
            except (TypeError, ValueError):
                pass
        elif kind == _J:
            cp.set(section, key, _dumps(v))
        elif kind in (_JN, _JA):
            if v is not None:
                cp.set(section, key, _dumps(np.asarray(v) if kind == _JA else v))
        elif kind == "dose":
            if np.any(v) and bool(reg.filterMode):
                cp.set(section, key, _dumps(v))
    for n, ed in enumerate(reg.errorDictList):
        name = "errorDict%d" % n
        cp.add_section(name)
        keys = list(ed.keys())
        cp.set(name, "keyList", json.dumps(keys))
        for k in keys:
            cp.set(name, k, _dumps(ed[k]))
    with open(path, "w+") as fh:
        cp.write(fh)
    return path


def _get(cp, section, key, how):
    if how == "int":
        return cp.getint(section, key)
    if how == "float":
        return cp.getfloat(section, key)
    if how == "bool":
        return cp.getboolean(section, key)
    if how == "upper":
        return cp.get(section, key).upper()
    if how == "json":
        return json.loads(cp.get(section, key))
    if how == "array":
        return np.array(json.loads(cp.get(section, key)))
    return cp.get(section, key)


def load_config(reg, configNameIn=None, loadData=False):
    """Set ``reg``'s attributes from a .zor file (zorro.py:3682-3887)."""
    if configNameIn:
        reg.files["config"] = configNameIn
    path = reg.files.get("config")
    if not path or not os.path.isfile(path):
        raise IOError("zorro.loadConfig: Could not load config file %s" % path)
    cp = _parser()
    cp.read(path)
    for item in _READS:
        if item == "errorDicts":
            n = 0
            while True:
                name = "errorDict%d" % n
                try:
                    ed = {}
                    for k in json.loads(cp.get(name, "keyList")):
                        v = np.array(json.loads(cp.get(name, k)))
                        ed[k] = v.item(0) if v.size == 1 else v
                except Exception:
                    break
                reg.errorDictList.append(ed)
                n += 1
            continue
        section, key, attr, how = item
        try:
            setattr(reg, attr, _get(cp, section, key, how))
        except Exception:
            pass
    if loadData and "stack" in reg.files and reg.files["stack"] is not None:
        reg.loadData()
    return reg

"""Drop-in ``ImageRegistrator`` whose ``alignImageStack`` runs on the GPU.

The class keeps the attribute names, defaults and outputs of
``zorro.ImageRegistrator`` (zorro/zorro.py:78-243) for the registration hot
path, and ``alignImageStack()`` (zorro.py:1569-1716) drives the sm_103a
kernels of ``libzorrogb.so`` through its C ABI.  PyTorch is used only to own
device buffers and the stream.  Nothing falls back to the CPU: without the
library or a CUDA device the call raises.

Inputs, as the reference holds them after ``loadData``:

* ``images``: [N,H,W] float32 (gain already applied), or raw detector counts
  (uint8/uint16/float16) together with ``gainRef`` ([H,W] float32, already
  oriented by ``gainInfo``), in which case the gain multiply of
  ``loadData`` (zorro.py:3466) is fused into every kernel that reads a frame.
  A CUDA ``torch.Tensor`` is accepted as well and stays on the device.
* the registration attributes below.

Outputs left on the object (as the reference leaves them): ``translations``,
``imageSum``, ``errorDictList[-1]``, ``FRC``/``FRC2D``, ``filtSum``,
``hotpixInfo``, ``peaksigThres``/``logisticK``/``logisticNu``,
``shapeOriginal`` and ``bench``.  The reference also leaves the shifted
frames in ``images``; here that happens when ``keepAlignedImages`` is True
(the default).
"""
from __future__ import annotations

import copy
import time

import numpy as np

from . import _lib
from . import hostmath as hm


class ImageRegistrator:
    """GPU drop-in for zorro.ImageRegistrator's registration path."""

    def __init__(self):
        # defaults of zorro.py:82-243 that the hot path reads
        self.verbose = 0
        self.METAstatus = "new"
        self.xcorrMode = "zorro"
        self.n_threads = None
        self.cachePath = None
        self.pixelsize = None
        self.voltage = 300.0
        self.C3 = 2.7
        self.gain = None
        self.bench = {}
        self.saveC = False
        self.Brad = 512
        self.Bmode = "opti"
        self.BfiltType = "gaussian"
        self.fouCrop = [3072, 3072]
        self.images = None
        self.imageSum = None
        self.filtSum = None
        self.gainRef = None
        self.gainInfo = {"Horizontal": True, "Vertical": True, "Diagonal": False,
                         "GammaParams": [0.12035633, -1.04171635, -0.03363192, 1.03902726]}
        self.filterMode = None
        self.doseFiltParam = [None, 0.24499, -1.6649, 2.8141, 32, 0]
        self.hotpixInfo = {"logisticK": 6.0, "relax": 0.925, "maxSigma": 8.0, "psf": "K2", "guessHotpix": 0,
                           "guessDeadpix": 0, "decorrOutliers": False, "cutoffLower": -4.0, "cutoffUpper": 3.25,
                           "neighborPix": 0}
        self.masks = None
        self.C = None
        self.translations = None
        self.errorDictList = []
        self.doLazyFRC = True
        self.doEvenOddFRC = False
        self.FRC = None
        self.FRC2D = None
        self.transEven = None   # half-set trajectories of doEvenOddFRC
        self.transOdd = None
        self.CTFProgram = None
        self.shapePadded = [4096, 4096]
        self.shapeOriginal = None
        self.shapeBinned = None
        self.subPixReg = 16
        self.shiftMethod = "lanczos"
        self.maxShift = 100
        self.preShift = False
        self.peakLocMode = "interpolated"
        self.weightMode = "autologistic"
        self.peaksigThres = 6.0
        self.logisticK = 5.0
        self.logisticNu = 0.15
        self.originMode = "centroid"
        self.suppressOrigin = True
        self.triMode = "diag"
        self.startFrame = 0
        self.endFrame = 0
        self.diagStart = 0
        self.diagWidth = 5
        self.autoMax = 10
        self.corrThres = None
        # GB300 build: options of the GPU path
        self.keepAlignedImages = True   # copy the shifted frames back into ``images``
        self.subtractFrameMean = True    # exact identity, see zorro_gb300.engine
        self.returnDeviceArrays = False  # leave imageSum/filtSum/FRC as CUDA tensors
        # 'float16': frame spectra stored in half precision with per-spectrum
        # power-of-two scales (products and transforms stay float32)
        self.spectraPrecision = "float32"
        self.device = 0

    def loadGainRef(self, gain):
        """Set ``gainRef`` from a gain-reference array as loadData does when it
        reads one (target 'gainRef', zorro.py:3486-3502): rotated by 90
        degrees if gainInfo['Diagonal'], then rotated by 180 degrees if both
        'Horizontal' and 'Vertical', else flipped left-right ('Horizontal')
        or up-down ('Vertical').  The multiply by the frames (zorro.py:3466)
        happens inside the kernels that read them."""
        g = np.asarray(gain, dtype=np.float32)
        info = self.gainInfo or {}
        if info.get("Diagonal"):
            g = np.rot90(g, k=1)
        if info.get("Horizontal") and info.get("Vertical"):
            g = np.rot90(g, k=2)
        elif info.get("Horizontal"):
            g = np.fliplr(g)
        elif info.get("Vertical"):
            g = np.flipud(g)
        self.gainRef = np.ascontiguousarray(g)
        return self.gainRef

    def alignImageStack(self):
        """Register and sum the stack.  zorro.py:1569-1716."""
        if str(self.xcorrMode).lower() != "zorro":
            raise ValueError("Zorro.alignImageStack: only xcorrMode 'zorro' runs on the GPU, not %s" % self.xcorrMode)
        from .engine import Engine
        Engine.get(self.device).align(self)


def copy_config(src, dst):
    """Copy the registration attributes of one registrator to another."""
    for k, v in vars(src).items():
        if k in ("images", "imageSum", "filtSum", "gainRef", "masks", "errorDictList", "FRC", "FRC2D",
                 "translations"):
            continue
        setattr(dst, k, copy.deepcopy(v))
    return dst

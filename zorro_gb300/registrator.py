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
import tempfile
import time

import numpy as np

from . import _lib
from . import hostmath as hm


class ImageRegistrator:
    """GPU drop-in for zorro.ImageRegistrator's registration path."""

    def __init__(self):
        # defaults of zorro.py:82-243 (the hot path's, and the rest of what
        # the .zor configs carry)
        self.verbose = 0
        self.umask = 2
        self.METApriority = 0.0
        self.METAstatus = "new"
        self.METAmtime = 0.0
        self.METAsize = 0
        self.xcorrMode = "zorro"
        self.fftw_effort = "FFTW_MEASURE"
        self.n_threads = None
        self.cachePath = tempfile.gettempdir()
        self.pixelsize = None
        self.voltage = 300.0
        self.C3 = 2.7
        self.gain = None
        self.detectorPixelSize = None
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
        self.velocities = None
        self.rotations = None
        self.scales = None
        self.errorDictList = []
        self.trackCorrStats = False
        self.corrStats = None
        self.doLazyFRC = True
        self.doEvenOddFRC = False
        self.FRC = None
        self.FRC2D = None
        self.transEven = None   # half-set trajectories of doEvenOddFRC
        self.transOdd = None
        # addition: the half-set registrations' error dictionaries of
        # doEvenOddFRC ({'even': ..., 'odd': ...}); the reference discards them
        self.halfSetErrorDicts = None
        self.CTFProgram = None
        self.CTFInfo = {"DefocusU": None, "DefocusV": None, "DefocusAngle": None, "CtfFigureOfMerit": None,
                        "FinalResolution": None, "AmplitudeContrast": 0.07, "AdditionalPhaseShift": None}
        self.CTFDiag = None
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
        self.velocityThres = None
        # input/output (zorro.py:218-230)
        self.files = {"config": None, "stack": None, "mask": None, "sum": None, "align": None, "figurePath": None,
                      "xc": None, "moveRawPath": None, "original": None, "gainRef": None, "stdout": None,
                      "automatch": None, "rejected": None, "compressor": None, "clevel": 1}
        self.savePNG = True
        self.saveMovie = True
        self.doCompression = False
        self.compress_ext = ".bz2"
        # plotting options (zorro.py:233-241): carried through the configs, no plots are drawn
        self.plotDict = {"imageSum": True, "imageFirst": False, "FFTSum": True, "polarFFTSum": True, "filtSum": True,
                         "stats": False, "corrTriMat": False, "peaksigTriMat": True, "translations": True,
                         "pixRegError": True, "CTFDiag": True, "logisticWeights": True, "FRC": True,
                         "Transparent": True, "plot_dpi": 144, "image_dpi": 250, "image_cmap": "gray",
                         "graph_cmap": "gnuplot", "fontsize": 12, "fontstyle": "serif", "colorbar": True,
                         "backend": "Qt4Agg", "multiprocess": True, "show": False}
        # GB300 build: options of the GPU path
        self.keepAlignedImages = True   # copy the shifted frames back into ``images``
        self.subtractFrameMean = True    # exact identity, see zorro_gb300.engine
        self.returnDeviceArrays = False  # leave imageSum/filtSum/FRC as CUDA tensors
        # float32 ``images`` from loadData still without gainRef / gain (the
        # kernels apply them as they read the frames)
        self.imagesAreRaw = False
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

    def loadData(self, stackNameIn=None, target="stack"):
        """Read an MRC file into ``target`` (zorro.py:3268-3516, MRC branch
        :3414-3425 and the gain / assignment steps :3455-3516).

        * The pixel size comes from the header when it is nonzero (nm), for
          every target: a gain reference read on behalf of a movie replaces
          the movie's pixel size when its own header has one, as in the
          reference.
        * Movies stay in their detector type (uint8, uint16, float16, float32,
          or the packed 4-bit ``mrc.Packed4``) in page-locked host memory,
          int8/int16 ones become float32; the gain reference multiply and the
          ``gain`` division that the reference applies here on the host run
          inside the kernels that read the frames (same float32 values).
          ``imagesAreRaw`` marks float32 frames that still need them.
        * target 'gainRef' orients the reference by ``gainInfo``
          (``loadGainRef``); 'sum'/'imageSum', 'filt'/'filtSum' and 'mask'
          set those attributes.

        DM4 files (``dm4.read``) give their second image and its calibration,
        voltage and Cs; MRCZ files are read by ``mrc.read`` (blosc-compressed
        slices).  DM3/TIFF/HDF5 and .bz2/.gz files are not read."""
        import os

        from . import mrc
        if stackNameIn is not None:
            self.files[target] = stackNameIn
        name = self.files.get(target)
        if not name:
            raise ValueError("zorro.loadData: no file for target %r" % target)
        ext = os.path.splitext(str(name))[1].lower()
        if ext == ".dm4":
            # zorro.py:3384-3411: the second image of the file (the first is
            # the thumbnail), its calibration (nm) unless it has no units, the
            # microscope's voltage (kV) and Cs
            from . import dm4
            data, info = dm4.read(name)
            if data.ndim == 2:
                data = data[None]
            if info["pixelsize"] is not None:
                self.pixelsize = info["pixelsize"]
            if info["voltage"]:
                self.voltage = info["voltage"]
            if info["C3"]:
                self.C3 = info["C3"]
        elif ext in (".mrc", ".mrcs", ".mrcz", ".mrczs"):
            data, hdr = mrc.read(name, pinned=target in ("stack", "align", "images"))
            if not np.isclose(hdr["pixelsize"][0], 0.0):
                self.pixelsize = np.float32(hdr["pixelsize"][0])
        else:
            raise ValueError("zorro.loadData: %s files are not supported (MRC, MRCZ or DM4)" % ext)
        if target in ("stack", "align", "images"):
            if data.ndim != 3 or data.shape[0] < 2:  # a single image, saved by mistake
                self.METAstatus = "error"
                raise ValueError("zorro.loadData: stacks must be 3D data")
            if target != "gainRef" and self.files.get("gainRef") and self.gainRef is None:
                self.loadData(self.files["gainRef"], target="gainRef")
            # gainRef and gain are applied as the kernels read the frames
            if isinstance(data, mrc.Packed4) or data.dtype in (np.uint8, np.uint16, np.float16, np.float32):
                self.images = data
            else:
                self.images = data.astype(np.float32)  # float32(int), as the reference's astype
            self.imagesAreRaw = not isinstance(data, mrc.Packed4) and self.images.dtype == np.float32
        elif target == "gainRef":
            if isinstance(data, mrc.Packed4):
                raise ValueError("zorro.loadData: a 4-bit gain reference is not supported")
            self.loadGainRef(data[0] if data.shape[0] == 1 else data)
        elif target in ("sum", "imageSum"):
            self.imageSum = np.asarray(data[0] if data.shape[0] == 1 else data, dtype=np.float32)
        elif target in ("filt", "filtSum"):
            self.filtSum = np.asarray(data[0] if data.shape[0] == 1 else data, dtype=np.float32)
        elif target == "mask":
            self.masks = np.asarray(data)
        else:
            raise ValueError("zorro.loadData: unknown target %r" % target)

    def saveData(self):
        """Write the aligned sum, the aligned movie (``saveMovie``) and the
        filtered sum as MRC files (zorro.py:3538-3627): default names
        sum/<stack>_zorro.mrc, align/<stack>_zorro_movie.mrcs and
        <sum>_filt.mrc next to the sum, pixel size in the header.  Compressed
        output (``files['compressor']``, ``doCompression``) is not written."""
        import os

        from . import mrc
        if self.files.get("compressor") or self.doCompression:
            raise ValueError("zorro.saveData: compressed output is not supported")
        stack = self.files.get("stack") or "stack.mrc"
        front, ext = os.path.splitext(os.path.basename(str(stack)))
        if ext in (".bz2", ".gz", ".7z"):
            front = os.path.splitext(front)[0]
        if self.files.get("sum") is None:
            self.files["sum"] = os.path.join("sum", "%s_zorro.mrc" % front)
        sum_path = self.files["sum"]
        mrc.write(sum_path, self._host(self.imageSum), pixelsize=self.pixelsize)
        if self.saveMovie and self.images is not None and not isinstance(self.images, mrc.Packed4):
            if self.files.get("align") is None:
                self.files["align"] = os.path.join("align", "%s_zorro_movie.mrcs" % front)
            mrc.write(self.files["align"], self._host(self.images), pixelsize=self.pixelsize)
        if self.filterMode and self.filtSum is not None:
            if self.files.get("filt") is None:
                self.files["filt"] = os.path.join(os.path.dirname(sum_path),
                                                  "%s_filt.mrc" % os.path.splitext(os.path.basename(sum_path))[0])
            mrc.write(self.files["filt"], self._host(self.filtSum), pixelsize=self.pixelsize)

    def saveConfig(self, configNameIn=None):
        """Write the state as a .zor file (zorro.py:3889-4075; zorro_gb300.config)."""
        from .config import save_config
        return save_config(self, configNameIn)

    def loadConfig(self, configNameIn=None, loadData=False):
        """Read a .zor file into the attributes (zorro.py:3682-3887;
        zorro_gb300.config), then the movie when ``loadData``."""
        from .config import load_config
        return load_config(self, configNameIn, loadData)

    @staticmethod
    def _host(a):
        if hasattr(a, "detach"):
            a = a.detach().cpu().numpy()
        return np.asarray(a)

    @property
    def masks(self):
        """The registration mask (None: the whole frame).  After a registration
        without one this is the all-true [1, H, W] mask the reference leaves
        (zorro.py:584-586), made when first read rather than for every
        movie."""
        m = self.__dict__.get("_masks")
        if m is None and self.__dict__.get("_ones_mask_shape") is not None:
            H, W = self._ones_mask_shape
            m = self._masks = np.ones([1, H, W], dtype=bool)
        return m

    @masks.setter
    def masks(self, v):
        self._masks = v
        self._ones_mask_shape = None

    def alignImageStack(self):
        """Register and sum the stack.  zorro.py:1569-1716."""
        if str(self.xcorrMode).lower() != "zorro":
            raise ValueError("Zorro.alignImageStack: only xcorrMode 'zorro' runs on the GPU, not %s" % self.xcorrMode)
        from .engine import Engine
        Engine.get(self.device).align(self)


def alignImageStacks(registrators, device=None):
    """Register several movies at once on one GPU: alignImageStack for each
    registrator (each keeps its own settings, detector size and frame count),
    with the transform-heavy stages of movies that share a shape class run
    as one set of launches (Engine.align_batch).  The outputs are those each
    registrator gets from alignImageStack alone.  Has no counterpart in the
    reference, which registers one movie per process."""
    regs = list(registrators)
    if not regs:
        return regs
    for r in regs:
        if str(r.xcorrMode).lower() != "zorro":
            raise ValueError("Zorro.alignImageStack: only xcorrMode 'zorro' runs on the GPU, not %s" % r.xcorrMode)
    from .engine import Engine
    dev = regs[0].device if device is None else device
    Engine.get(dev).align_batch(regs)
    return regs


def copy_config(src, dst):
    """Copy the registration attributes of one registrator to another."""
    for k, v in vars(src).items():
        if k in ("images", "imageSum", "filtSum", "gainRef", "masks", "_masks", "_ones_mask_shape", "errorDictList",
                 "FRC", "FRC2D", "translations", "files", "imagesAreRaw"):
            continue
        setattr(dst, k, copy.deepcopy(v))
    return dst

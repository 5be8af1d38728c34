"""ctypes binding of ``libzorrogb.so`` (declarations in include/zorro_gb300.h).

Loading fails loudly when the library is missing: there is no CPU fallback
for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libzorrogb.so")

ZR_F32, ZR_U8, ZR_U16, ZR_F16 = 0, 1, 2, 3

# every symbol the header declares
EXPORTS = (
    "zr_version", "zr_last_error", "zr_launch_count", "zr_init", "zr_gain_sum", "zr_histogram", "zr_hotpix_thresholds",
    "zr_hotpix_work_bytes",
    "zr_hotpix_maps", "zr_frame_sums", "zr_spectrum_pitch", "zr_spectrum_elems", "zr_spectra_work_bytes",
    "zr_spectra", "zr_xcorr_work_bytes", "zr_xcorr_terms", "zr_xcorr_pairs", "zr_locate_peaks",
    "zr_shift_sum", "zr_frc_work_bytes", "zr_tiled_frc", "zr_dose_work_bytes", "zr_dose_filter",
    "zr_l1_solve", "zr_xcorr_pairs_noalloc", "zr_logistic_fit", "zr_refine_spectra", "zr_refine_terms",
    "zr_xcorr_refine", "zr_pack_half", "zr_xcorr_terms_half", "zr_xcorr_pairs_half", "zr_bin_work_bytes",
    "zr_bin_fourier", "zr_unpack_u4", "zr_full_prepare", "zr_full_work_bytes", "zr_full_filter", "zr_full_peaks",
    "zr_plan_work_bytes", "zr_plan", "zr_plan_set", "zr_plan_get", "zr_lz4_decompress",
    "zr_ctx_create", "zr_ctx_destroy", "zr_submit_batch", "zr_poll", "zr_wait",
)


class Frames(C.Structure):
    """zr_frames_t.  ``frame_movie``/``map_stride`` (the batched path) stay
    zero unless frames of several movies share a call."""
    _fields_ = [("raw", C.c_void_p), ("raw_type", C.c_int), ("gain", C.c_void_p), ("hot_a", C.c_void_p),
                ("hot_b", C.c_void_p), ("gain_divisor", C.c_float), ("n_frames", C.c_int), ("height", C.c_int),
                ("width", C.c_int), ("frame_stride", C.c_longlong), ("frame_movie", C.c_void_p),
                ("map_stride", C.c_longlong)]


class HotpixParams(C.Structure):
    _fields_ = [("mu", C.c_double), ("sigma", C.c_double), ("cutoff_lower", C.c_float),
                ("cutoff_upper", C.c_float), ("logistic_k", C.c_float), ("relax", C.c_float),
                ("psf", C.c_float * 9), ("neighbour_thres", C.c_float), ("best_mean", C.c_double)]


class PeakParams(C.Structure):
    _fields_ = [("sub_pix_reg", C.c_int), ("bmode", C.c_int), ("suppress_origin", C.c_int), ("use_mask", C.c_int),
                ("conv_sigma_y", C.c_double), ("conv_sigma_x", C.c_double), ("opti_lo", C.c_double),
                ("opti_hi", C.c_double), ("opti_xatol", C.c_double), ("opti_maxiter", C.c_int)]


class PeakResult(C.Structure):
    _fields_ = [("shift_y", C.c_double), ("shift_x", C.c_double), ("sigma", C.c_double), ("corr", C.c_float),
                ("peaksig", C.c_float), ("origin", C.c_float), ("cy", C.c_int), ("cx", C.c_int),
                ("flags", C.c_int), ("nfev", C.c_int)]


class PlanShape(C.Structure):
    _fields_ = [("P0", C.c_int), ("P1", C.c_int), ("C0", C.c_int), ("C1", C.c_int), ("max_shift", C.c_int),
                ("n_frames", C.c_int)]


class PlanChoice(C.Structure):
    _fields_ = [("fwd_rows", C.c_int), ("fwd_cols", C.c_int), ("xc_cols", C.c_int), ("xc_rows", C.c_int),
                ("ms_spectra", (C.c_float * 3) * 3), ("ms_pairs", (C.c_float * 3) * 3)]


class BatchLimits(C.Structure):
    """zr_batch_limits_t: one shape class and the most frames and pairs of a
    batch."""
    _fields_ = [("height", C.c_int), ("width", C.c_int), ("P0", C.c_int), ("P1", C.c_int), ("C0", C.c_int),
                ("C1", C.c_int), ("max_shift", C.c_int), ("max_frames", C.c_int), ("max_pairs", C.c_int),
                ("chunk_frames", C.c_int)]


class BatchMovie(C.Structure):
    """zr_batch_movie_t: one movie of a batch (pairs and peaks in host
    memory)."""
    _fields_ = [("frames", Frames), ("mean_sub", C.c_void_p), ("pairs", C.c_void_p), ("n_pairs", C.c_int),
                ("peaks", C.c_void_p)]


class Shift(C.Structure):
    _fields_ = [("roll_y", C.c_int), ("roll_x", C.c_int), ("apply", C.c_int), ("ky", C.c_float * 3),
                ("kx", C.c_float * 3)]


class DoseParams(C.Structure):
    _fields_ = [("crit_a", C.c_float), ("crit_b", C.c_float), ("crit_c", C.c_float), ("cutoff_order", C.c_float),
                ("voltage_scaling", C.c_float), ("inv_ps_x", C.c_float), ("inv_ps_y", C.c_float),
                ("normalize", C.c_int)]


class ZorroError(RuntimeError):
    pass


_lib = None

_P = C.c_void_p
_SIGS = {
    "zr_version": (C.c_int, []),
    "zr_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
    "zr_launch_count": (C.c_ulonglong, []),
    "zr_init": (C.c_int, [C.c_int]),
    "zr_gain_sum": (C.c_int, [C.POINTER(Frames), _P, _P, _P]),
    "zr_histogram": (C.c_int, [_P, C.c_longlong, C.c_double, C.c_int, _P, _P]),
    "zr_hotpix_thresholds": (C.c_int, [C.c_double, C.c_double, C.c_float, C.c_float, C.POINTER(C.c_float),
                                       C.POINTER(C.c_float)]),
    "zr_hotpix_work_bytes": (C.c_size_t, [C.c_int, C.c_int]),
    "zr_hotpix_maps": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.POINTER(HotpixParams), _P, _P, _P, _P,
                                 C.c_size_t, _P]),
    "zr_frame_sums": (C.c_int, [C.POINTER(Frames), _P, _P]),
    "zr_spectrum_pitch": (C.c_int, [C.c_int]),
    "zr_spectrum_elems": (C.c_longlong, [C.c_int, C.c_int]),
    "zr_spectra_work_bytes": (C.c_size_t, [C.c_int, C.c_int, C.c_int]),
    "zr_spectra": (C.c_int, [C.POINTER(Frames), _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                             C.c_int, _P, _P, _P, C.c_size_t, _P]),
    "zr_xcorr_work_bytes": (C.c_size_t, [C.c_int, C.c_int, C.c_int]),
    "zr_xcorr_terms": (C.c_int, [_P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P, C.c_size_t, _P]),
    "zr_xcorr_pairs": (C.c_int, [_P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P, C.c_size_t,
                                 _P]),
    "zr_bin_work_bytes": (C.c_size_t, [C.c_int, C.c_int, C.c_int, C.c_int]),
    "zr_bin_fourier": (C.c_int, [C.POINTER(Frames), C.c_int, C.c_int, _P, _P, C.c_size_t, _P]),
    "zr_unpack_u4": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _P, _P]),
    "zr_full_prepare": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _P, _P, _P]),
    "zr_full_work_bytes": (C.c_size_t, [C.c_int, C.c_int]),
    "zr_full_filter": (C.c_int, [_P, C.c_int, C.c_int, _P, C.c_int, _P, _P, _P, _P, _P, _P, C.c_size_t, _P]),
    "zr_full_peaks": (C.c_int, [_P, _P, C.c_int, C.c_int, _P, C.c_int, C.c_int, _P, _P, _P, _P, _P, C.c_int, _P, _P,
                                C.c_size_t, _P]),
    "zr_pack_half": (C.c_int, [_P, C.c_int, C.c_longlong, _P, _P, _P, C.c_size_t, _P]),
    "zr_xcorr_terms_half": (C.c_int, [_P, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P, C.c_size_t, _P]),
    "zr_xcorr_pairs_half": (C.c_int, [_P, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P,
                                      C.c_size_t, _P]),
    "zr_refine_spectra": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _P, _P]),
    "zr_refine_terms": (C.c_int, [_P, C.c_int, C.c_int, _P, _P]),
    "zr_xcorr_refine": (C.c_int, [_P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P, C.c_size_t, _P]),
    "zr_logistic_fit": (C.c_int, [_P, _P, C.c_int, _P, _P, _P, C.c_double, C.c_double, C.c_int, C.c_int, _P, _P,
                                  _P]),
    "zr_xcorr_pairs_noalloc": (C.c_int, [_P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P]),
    "zr_locate_peaks": (C.c_int, [_P, C.c_int, C.c_int, C.POINTER(PeakParams), _P, _P]),
    "zr_shift_sum": (C.c_int, [C.POINTER(Frames), _P, _P, _P, _P, _P, _P]),
    "zr_frc_work_bytes": (C.c_size_t, [C.c_int, C.c_int]),
    "zr_tiled_frc": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, _P, C.c_int, _P, _P, C.c_int, _P, C.c_size_t,
                               _P]),
    "zr_dose_work_bytes": (C.c_size_t, [C.c_int, C.c_int, C.c_int]),
    "zr_l1_solve": (C.c_int, [_P, _P, _P, C.c_int, C.c_int, C.c_double, C.c_double, _P, C.POINTER(C.c_int)]),
    "zr_dose_filter": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.POINTER(DoseParams), _P, _P, C.c_int, C.c_int,
                                 _P, _P, C.c_size_t, _P]),
    "zr_plan_work_bytes": (C.c_size_t, [C.POINTER(PlanShape)]),
    "zr_plan": (C.c_int, [C.POINTER(PlanShape), _P, C.c_size_t, _P, C.POINTER(PlanChoice)]),
    "zr_plan_set": (C.c_int, [C.POINTER(PlanShape), C.POINTER(PlanChoice)]),
    "zr_plan_get": (C.c_int, [C.POINTER(PlanShape), C.POINTER(PlanChoice)]),
    "zr_lz4_decompress": (C.c_longlong, [_P, C.c_size_t, _P, C.c_size_t]),
    "zr_ctx_create": (C.c_int, [C.c_int, C.POINTER(BatchLimits), C.POINTER(C.c_void_p)]),
    "zr_ctx_destroy": (C.c_int, [_P]),
    "zr_submit_batch": (C.c_int, [_P, _P, C.c_int, C.POINTER(PeakParams), _P]),
    "zr_poll": (C.c_int, [_P]),
    "zr_wait": (C.c_int, [_P]),
}


def load(path=None):
    """Load the library (once).  Raises when it is missing or incomplete."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("ZORRO_GB300_LIB") or LIB_PATH
    if not os.path.exists(path):
        raise ZorroError("libzorrogb.so not found at %s: build it with `python -m zorro_gb300.build` "
                         "(there is no CPU fallback)" % path)
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error():
    buf = C.create_string_buffer(512)
    load().zr_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(rc, what):
    if rc != 0:
        msg = "%s failed (code %d): %s" % (what, rc, last_error())
        if rc in (-1, -3):
            raise ValueError(msg)
        raise ZorroError(msg)
    return rc


def call(name, *args):
    return check(getattr(load(), name)(*args), name)

"""Stage-by-stage calls of libzorrogb through its C ABI, for the GPU tests."""
import ctypes as C

import numpy as np

from zorro_gb300 import _lib
from zorro_gb300._lib import Frames, PeakParams, PeakResult

PEAK_DTYPE = np.dtype([("sy", "f8"), ("sx", "f8"), ("sigma", "f8"), ("corr", "f4"), ("peaksig", "f4"),
                       ("origin", "f4"), ("cy", "i4"), ("cx", "i4"), ("flags", "i4"), ("nfev", "i4")], align=True)


def torch_mod():
    import torch
    return torch


def dev_tensor(a):
    torch = torch_mod()
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def stream():
    return torch_mod().cuda.current_stream().cuda_stream


def frames_of(raw_t, gain_t=None):
    N, H, W = raw_t.shape
    rtype = {np.dtype(np.float32): _lib.ZR_F32, np.dtype(np.uint8): _lib.ZR_U8,
             np.dtype(np.uint16): _lib.ZR_U16}[np.dtype(str(raw_t.dtype).replace("torch.", ""))]
    return Frames(raw_t.data_ptr(), rtype, gain_t.data_ptr() if gain_t is not None else None, None, None, 0.0,
                  N, H, W, 0)


def spectra(images, P, C_, mean_sub=True):
    """(G, S, GM) as complex128 numpy arrays [N, C0+1, K4], [N, ...], [C0+1, K4]."""
    torch = torch_mod()
    lib = _lib.load()
    _lib.call("zr_init", torch.cuda.current_device())
    raw = dev_tensor(images.astype(np.float32))
    N, H, W = images.shape
    fr = frames_of(raw)
    se = lib.zr_spectrum_elems(C_[0], C_[1])
    K4 = lib.zr_spectrum_pitch(C_[1])
    G = torch.zeros((N, se, 2), dtype=torch.float32, device="cuda")
    S = torch.zeros((N, se, 2), dtype=torch.float32, device="cuda")
    GM = torch.zeros((se, 2), dtype=torch.float32, device="cuda")
    wb = lib.zr_spectra_work_bytes(H, N, C_[1])
    work = torch.empty(wb, dtype=torch.uint8, device="cuda")
    msub = None
    if mean_sub:
        msub = torch.zeros(N, dtype=torch.float64, device="cuda")
        _lib.call("zr_frame_sums", C.byref(fr), msub.data_ptr(), stream())
    _lib.call("zr_spectra", C.byref(fr), None, None, 0, 1, 1, P[0], P[1], C_[0], C_[1], GM.data_ptr(), None,
              work.data_ptr(), wb, stream())
    _lib.call("zr_spectra", C.byref(fr), None, msub.data_ptr() if msub is not None else None, 0, N, 0, P[0], P[1],
              C_[0], C_[1], G.data_ptr(), S.data_ptr(), work.data_ptr(), wb, stream())
    torch.cuda.synchronize()

    def cx(t, n):
        # column-major [K4][C0+4] -> [C0+1][K4]
        a = t.cpu().numpy().astype(np.float64)
        a = (a[..., 0] + 1j * a[..., 1]).reshape(n, K4, C_[0] + 4)[:, :, :C_[0] + 1]
        return np.swapaxes(a, 1, 2)

    means = (msub.cpu().numpy() / (H * W)) if msub is not None else np.zeros(N)
    return (cx(G, N), cx(S, N), cx(GM, 1)[0], means, (G, S, GM))


def windows(dev_spectra, N, C_, mS, pairs):
    torch = torch_mod()
    lib = _lib.load()
    G, S, GM = dev_spectra
    w = 2 * mS
    terms = torch.zeros((4 * N + 1, w, w), dtype=torch.float32, device="cuda")
    M = len(pairs)
    xw = lib.zr_xcorr_work_bytes(7, C_[1], mS)  # small waves on purpose
    work = torch.empty(xw, dtype=torch.uint8, device="cuda")
    _lib.call("zr_xcorr_terms", G.data_ptr(), S.data_ptr(), GM.data_ptr(), N, C_[0], C_[1], mS, terms.data_ptr(),
              work.data_ptr(), xw, stream())
    pd = dev_tensor(np.asarray(pairs, dtype=np.int32).reshape(-1))
    cwin = torch.zeros((M, w, w), dtype=torch.float32, device="cuda")
    _lib.call("zr_xcorr_pairs", G.data_ptr(), terms.data_ptr(), pd.data_ptr(), M, N, C_[0], C_[1], mS,
              cwin.data_ptr(), work.data_ptr(), xw, stream())
    torch.cuda.synchronize()
    return terms.cpu().numpy(), cwin.cpu().numpy(), cwin


def peaks(cwin_dev, mS, subPixReg=16, bmode=1, suppress=True):
    torch = torch_mod()
    M = cwin_dev.shape[0]
    pp = PeakParams()
    pp.sub_pix_reg = subPixReg
    pp.bmode = bmode
    pp.suppress_origin = int(suppress)
    pp.use_mask = 1
    pp.opti_lo, pp.opti_hi, pp.opti_xatol, pp.opti_maxiter = 0.0, 7.0, 0.01, 15
    out = torch.zeros((M, C.sizeof(PeakResult)), dtype=torch.uint8, device="cuda")
    _lib.call("zr_locate_peaks", cwin_dev.data_ptr(), M, mS, C.byref(pp), out.data_ptr(), stream())
    torch.cuda.synchronize()
    return np.frombuffer(out.cpu().numpy().tobytes(), dtype=PEAK_DTYPE)

"""zr_xcorr_pairs_noalloc (static scratch, no work buffer) against
zr_xcorr_pairs (caller's work buffer), through the C ABI.  The file name
sorts last so that the test also runs after every other GPU test."""
import ctypes as C

import numpy as np
import pytest

from tests import gpu_helpers as gh
from zorro_gb300 import _lib
from zorro_gb300.synthetic import make_movie

pytestmark = pytest.mark.gpu

# (frames, frame shape, padded, crop, maxShift)
CASES = [(6, (200, 180), (256, 256), (128, 128), 20),
         (5, (900, 1000), (1024, 1024), (1024, 1024), 100),
         (12, (1500, 1400), (2048, 2048), (2048, 2048), 100)]  # 66 pairs of 1,644,800 bytes: 7 waves of 10


@pytest.mark.parametrize("n,shape,P,C_,mS", CASES)
def test_noalloc_pairs_match_work_buffer_pairs(n, shape, P, C_, mS):
    torch = gh.torch_mod()
    lib = _lib.load()
    mv = make_movie(n, shape, seed=7, mean_dose=1.5, drift_sigma=1.0)
    _, _, _, _, dev = gh.spectra(mv["images"], P, C_)
    G, S, GM = dev
    w = 2 * mS
    terms = torch.zeros((4 * n + 1, w, w), dtype=torch.float32, device="cuda")
    xw = lib.zr_xcorr_work_bytes(4 * n + 1, C_[1], mS)
    work = torch.empty(xw, dtype=torch.uint8, device="cuda")
    _lib.call("zr_xcorr_terms", G.data_ptr(), S.data_ptr(), GM.data_ptr(), n, C_[0], C_[1], mS, terms.data_ptr(),
              work.data_ptr(), xw, gh.stream())
    pairs = np.array([(i, j) for i in range(n) for j in range(i + 1, n)], dtype=np.int32)
    M = len(pairs)
    pd = gh.dev_tensor(pairs.reshape(-1))
    ref = torch.zeros((M, w, w), dtype=torch.float32, device="cuda")
    pw = lib.zr_xcorr_work_bytes(M, C_[1], mS)
    pwork = torch.empty(pw, dtype=torch.uint8, device="cuda")
    _lib.call("zr_xcorr_pairs", G.data_ptr(), terms.data_ptr(), pd.data_ptr(), M, n, C_[0], C_[1], mS,
              ref.data_ptr(), pwork.data_ptr(), pw, gh.stream())
    torch.cuda.synchronize()
    ref_np = ref.cpu().numpy()
    assert np.isfinite(ref_np).all()
    for _ in range(2):  # two calls in a row reuse the one static scratch
        out = torch.full((M, w, w), np.nan, dtype=torch.float32, device="cuda")
        _lib.call("zr_xcorr_pairs_noalloc", G.data_ptr(), terms.data_ptr(), pd.data_ptr(), M, n, C_[0], C_[1], mS,
                  out.data_ptr(), gh.stream())
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.cpu().numpy(), ref_np, rtol=1e-6, atol=1e-7)


def test_noalloc_rejects_bad_arguments():
    lib = _lib.load()
    _lib.call("zr_init", 0)
    rc = lib.zr_xcorr_pairs_noalloc(None, None, None, 1, 2, 128, 128, 20, None, None)
    assert rc == -1
    assert "null" in _lib.last_error()
    torch = gh.torch_mod()
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    # a crop the kernels do not take: the same ZR_ESIZE as zr_xcorr_pairs
    rc = lib.zr_xcorr_pairs_noalloc(p, p, p, 1, 2, 8192, 8192, 20, p, None)
    assert rc == -3
    assert "crop" in _lib.last_error()
    # maxShift below 2: ZR_ESIZE, as zr_xcorr_pairs returns
    for ms in (0, 1):
        rc = lib.zr_xcorr_pairs_noalloc(p, p, p, 1, 2, 128, 128, ms, p, None)
        assert rc == -3, ms
        assert "maxShift" in _lib.last_error()
    # valid sizes whose one pair (1200 rows x 2052 columns x 8 bytes = 19.7 MB)
    # does not fit the 16 MiB array
    rc = lib.zr_xcorr_pairs_noalloc(p, p, p, 1, 2, 4096, 4096, 600, p, None)
    assert rc == -3
    assert "static scratch" in _lib.last_error()

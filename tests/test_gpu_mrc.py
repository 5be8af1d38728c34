"""Movie input on the GPU: the 4-bit unpack kernel (zr_unpack_u4) against the
oracle's restatement of MRC mode 101, and registrations of movies read from
MRC files (zorro.loadData, zorro.py:3414-3516) against the same movies given
as arrays."""
import ctypes as C

import numpy as np
import pytest

from oracle import mrc_oracle as mo
from zorro_gb300 import _lib
from zorro_gb300.registrator import ImageRegistrator
from zorro_gb300.synthetic import make_movie

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [(1, 1, 1), (1, 1, 2), (1, 3, 10), (3, 5, 9), (2, 7, 64), (4, 37, 3710)])
def test_unpack_u4_matches_oracle(shape):
    import torch
    rng = np.random.default_rng(sum(shape))
    pix = rng.integers(0, 16, size=shape).astype(np.uint8)
    packed = mo.pack4(pix)
    dp = torch.from_numpy(packed).cuda()
    out = torch.full(shape, 255, dtype=torch.uint8, device="cuda")
    _lib.call("zr_unpack_u4", dp.data_ptr(), shape[0], shape[1], shape[2], out.data_ptr(),
              C.c_void_p(torch.cuda.current_stream().cuda_stream))
    got = out.cpu().numpy()
    assert np.array_equal(got, mo.unpack4(packed, shape[2]))
    assert np.array_equal(got, pix)


def test_unpack_u4_rejects_bad_arguments():
    with pytest.raises(ValueError):
        _lib.call("zr_unpack_u4", None, 1, 1, 2, None, None)


ATTRS = dict(triMode="diag", diagWidth=3, shapePadded=[256, 256], fouCrop=[256, 256], maxShift=24,
             filterMode="hot")


def _align_file(path, gain_path=None, **kw):
    reg = ImageRegistrator()
    for k, v in {**ATTRS, **kw}.items():
        setattr(reg, k, v)
    if gain_path:
        reg.files["gainRef"] = gain_path
        reg.gainInfo = {"Horizontal": False, "Vertical": False, "Diagonal": False}
    reg.loadData(path)
    reg.alignImageStack()
    return reg


def test_four_bit_movie_registers_like_its_bytes(tmp_path):
    mv = make_movie(16, (256, 240), seed=5, mean_dose=1.6, drift_sigma=0.8, dtype="uint8", gain_map=True,
                    hot_fraction=1e-3)
    raw = np.minimum(mv["raw"], 15).astype(np.uint8)  # 4-bit counting frames saturate at 15
    p4 = mo.write(str(tmp_path / "m4.mrc"), raw, 101, pixelsize_nm=0.105)
    p8 = mo.write(str(tmp_path / "m8.mrc"), raw, 0, pixelsize_nm=0.105)
    pg = mo.write(str(tmp_path / "gain.mrc"), mv["gain"][None], 2, pixelsize_nm=0.0)
    a = _align_file(p4, pg)
    b = _align_file(p8, pg)
    assert a.pixelsize == b.pixelsize == np.float32(0.105)
    # the same uint8 frames reach the kernels: identical results
    assert np.array_equal(a.translations, b.translations)
    assert np.array_equal(a.imageSum, b.imageSum)
    for k in ("guessDeadpix", "guessHotpix", "neighborPix"):
        assert a.hotpixInfo[k] == b.hotpixInfo[k]
    # and the same as the in-memory registration of those counts with the gain
    c = ImageRegistrator()
    for k, v in ATTRS.items():
        setattr(c, k, v)
    c.pixelsize = np.float32(0.105)
    c.images = raw
    c.gainRef = mv["gain"]
    c.alignImageStack()
    assert np.array_equal(a.translations, c.translations)
    assert np.array_equal(a.imageSum, c.imageSum)


def test_float_movie_gain_applied_once(tmp_path):
    mv = make_movie(8, (128, 120), seed=9, mean_dose=2.0, drift_sigma=0.6, dtype="uint8", gain_map=True)
    frames = mv["raw"].astype(np.float32)
    pf = mo.write(str(tmp_path / "f.mrc"), frames, 2, pixelsize_nm=0.1)
    pg = mo.write(str(tmp_path / "g.mrc"), mv["gain"][None], 2, pixelsize_nm=0.0)
    attrs = dict(triMode="tri", shapePadded=[128, 128], fouCrop=[128, 128], maxShift=16)
    reg = ImageRegistrator()
    for k, v in attrs.items():
        setattr(reg, k, v)
    reg.gain = 1.25
    reg.files["gainRef"] = pg
    reg.gainInfo = {"Horizontal": True, "Vertical": False, "Diagonal": False}
    reg.loadData(pf)
    assert reg.imagesAreRaw and np.array_equal(reg.images, frames)
    reg.alignImageStack()
    assert not reg.imagesAreRaw
    # the frames the reference's loadData would hold: float32(gain * raw) / gain
    want = (np.fliplr(mv["gain"]).astype(np.float32) * frames) / np.float32(1.25)
    ref = ImageRegistrator()
    for k, v in attrs.items():
        setattr(ref, k, v)
    ref.images = want
    ref.alignImageStack()
    assert np.array_equal(reg.translations, ref.translations)
    assert np.array_equal(reg.imageSum, ref.imageSum)

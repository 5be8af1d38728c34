"""MRC movie input and sum output (zorro.loadData / saveData through mrcz,
zorro.py:3414-3425, 3573-3627) against the NumPy restatement of the format in
oracle/mrc_oracle.py.  CPU only: reading, writing and the host side of
loadData / saveData."""
import os
import struct

import numpy as np
import pytest

from oracle import mrc_oracle as mo
from zorro_gb300 import mrc
from zorro_gb300.registrator import ImageRegistrator

MODES = [(0, np.uint8, False), (0, np.int8, True), (1, np.int16, False), (2, np.float32, False),
         (4, np.complex64, False), (6, np.uint16, False), (12, np.float16, False)]


def _values(dtype, shape, rng):
    if dtype == np.complex64:
        return (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(np.complex64)
    if np.issubdtype(dtype, np.integer):
        info = np.iinfo(dtype)
        return rng.integers(info.min, int(info.max) + 1, size=shape).astype(dtype)
    return rng.normal(0, 100, size=shape).astype(dtype)


def test_packed4_known_answer(tmp_path):
    # two pixels a byte, the first in the low nibble; odd rows padded to a byte
    pix = np.array([[[1, 2, 3, 4, 5], [15, 0, 7, 8, 9]]], dtype=np.uint8)
    assert mo.pack4(pix).tolist() == [[[0x21, 0x43, 0x05], [0x0F, 0x87, 0x09]]]
    p = mo.write(str(tmp_path / "k.mrc"), pix, 101, pixelsize_nm=0.105)
    raw = open(p, "rb").read()
    assert raw[1024:] == bytes([0x21, 0x43, 0x05, 0x0F, 0x87, 0x09])
    data, h = mrc.read(p)
    assert isinstance(data, mrc.Packed4) and data.shape == (1, 2, 5)
    assert data.data.tolist() == [[[0x21, 0x43, 0x05], [0x0F, 0x87, 0x09]]]
    assert mo.unpack4(data.data, 5).tolist() == pix.tolist()
    assert h["mode"] == 101 and abs(h["pixelsize"][0] - 0.105) < 1e-6


def test_header_fields_known_answer(tmp_path):
    # a header written word by word: 7 x 3 x 2 float32, cell 14 A -> 2 A/px
    hdr = bytearray(1024)
    struct.pack_into("<10i", hdr, 0, 7, 3, 2, 2, 0, 0, 0, 7, 3, 2)
    struct.pack_into("<3f", hdr, 40, 14.0, 6.0, 4.0)
    struct.pack_into("<i", hdr, 92, 16)           # 16 bytes of extended header
    hdr[208:212] = b"MAP "
    hdr[212:214] = b"\x44\x44"
    body = np.arange(42, dtype="<f4")
    p = tmp_path / "h.mrc"
    p.write_bytes(bytes(hdr) + b"\xff" * 16 + body.tobytes())
    data, h = mrc.read(str(p))
    assert data.shape == (2, 3, 7) and data.dtype == np.float32
    assert np.array_equal(data.ravel(), body)
    assert h["pixelsize_A"] == (2.0, 2.0, 2.0) and abs(h["pixelsize"][0] - 0.2) < 1e-12
    # no IMOD stamp: mode-0 bytes are signed
    struct.pack_into("<i", hdr, 12, 0)
    p.write_bytes(bytes(hdr) + b"\x00" * 16 + bytes(range(200, 242)))
    d0, _ = mrc.read(str(p))
    assert d0.dtype == np.int8 and d0.ravel()[0] == 200 - 256


@pytest.mark.parametrize("order", ["<", ">"])
@pytest.mark.parametrize("mode,dtype,signed", MODES)
def test_read_matches_oracle_writer(tmp_path, mode, dtype, signed, order):
    rng = np.random.default_rng(mode + 7)
    a = _values(dtype, (3, 5, 9), rng)
    p = mo.write(str(tmp_path / "a.mrc"), a, mode, pixelsize_nm=0.0525, order=order, signed_bytes=signed,
                 nsymbt=64)
    data, h = mrc.read(p)
    ref, _, ps = mo.read(p)
    assert data.dtype == ref.dtype == np.dtype(dtype)
    assert np.array_equal(data, ref) and np.array_equal(data, a)
    assert abs(h["pixelsize"][0] - ps) < 1e-9 and abs(ps - 0.0525) < 1e-6
    assert h["byteorder"] == order


@pytest.mark.parametrize("nx", [8, 9, 3710])
def test_read_mode101_matches_oracle(tmp_path, nx):
    rng = np.random.default_rng(nx)
    pix = rng.integers(0, 16, size=(2, 4, nx)).astype(np.uint8)
    p = mo.write(str(tmp_path / "u4.mrc"), pix, 101)
    data, h = mrc.read(p)
    ref, _, _ = mo.read(p)
    assert np.array_equal(ref, pix)
    assert np.array_equal(data.data, mo.pack4(pix)) and data.shape == pix.shape


@pytest.mark.parametrize("mode,dtype,signed", MODES)
def test_writer_matches_oracle_reader(tmp_path, mode, dtype, signed):
    rng = np.random.default_rng(11 + mode)
    a = _values(dtype, (2, 6, 5), rng)
    p = mrc.write(str(tmp_path / "w.mrc"), a, pixelsize=0.105)
    ref, h, ps = mo.read(p)
    assert int(h["mode"]) == mode and ref.dtype == np.dtype(dtype)
    assert np.array_equal(ref, a) and abs(ps - 0.105) < 1e-6
    back, _ = mrc.read(p)
    assert np.array_equal(back, a)


def test_write_packed4_and_2d(tmp_path):
    pix = np.random.default_rng(3).integers(0, 16, size=(2, 3, 7)).astype(np.uint8)
    packed = mrc.Packed4(mo.pack4(pix), pix.shape)
    p = mrc.write(str(tmp_path / "p.mrc"), packed)
    ref, h, _ = mo.read(p)
    assert int(h["mode"]) == 101 and np.array_equal(ref, pix)
    img = np.random.default_rng(4).normal(size=(5, 6)).astype(np.float64)
    p2 = mrc.write(str(tmp_path / "s.mrc"), img)
    ref2, _, _ = mo.read(p2)
    assert ref2.shape == (1, 5, 6) and np.array_equal(ref2[0], img.astype(np.float32))


def test_bad_files(tmp_path):
    pix = np.zeros((1, 2, 4), np.uint8)
    p = mo.write(str(tmp_path / "t.mrc"), pix, 0)
    raw = open(p, "rb").read()
    (tmp_path / "short.mrc").write_bytes(raw[:-3])
    with pytest.raises(ValueError, match="truncated"):
        mrc.read(str(tmp_path / "short.mrc"))
    (tmp_path / "tiny.mrc").write_bytes(raw[:100])
    with pytest.raises(ValueError, match="header"):
        mrc.read(str(tmp_path / "tiny.mrc"))
    with pytest.raises(ValueError, match="compressed"):
        mrc.read(str(tmp_path / "t.mrc.gz"))
    bad = bytearray(raw)
    struct.pack_into("<i", bad, 12, 3)  # mode 3 (complex int16) is not a movie mode
    (tmp_path / "m3.mrc").write_bytes(bytes(bad))
    with pytest.raises(ValueError, match="mode 3"):
        mrc.read(str(tmp_path / "m3.mrc"))


def test_load_data_raw_movie_and_gain(tmp_path):
    rng = np.random.default_rng(5)
    raw = rng.integers(0, 6, size=(4, 6, 8)).astype(np.uint8)
    gain = rng.uniform(0.9, 1.1, size=(6, 8)).astype(np.float32)
    mo.write(str(tmp_path / "movie.mrc"), raw, 0, pixelsize_nm=0.105)
    mo.write(str(tmp_path / "gain.mrc"), gain[None], 2, pixelsize_nm=0.0)  # no pixel size in the gain header
    reg = ImageRegistrator()
    reg.files["gainRef"] = str(tmp_path / "gain.mrc")
    reg.gainInfo = {"Horizontal": True, "Vertical": True, "Diagonal": False}
    reg.loadData(str(tmp_path / "movie.mrc"))
    # raw counts kept (the gain multiply runs in the kernels), gain oriented
    assert reg.images.dtype == np.uint8 and np.array_equal(reg.images, raw)
    assert np.array_equal(reg.gainRef, np.rot90(gain, 2))
    assert reg.pixelsize == np.float32(0.105)
    assert reg.files["stack"] == str(tmp_path / "movie.mrc")
    # as in the reference, the gain reference is read by the same loadData,
    # so a pixel size in its header replaces the movie's (zorro.py:3422-3424)
    mo.write(str(tmp_path / "gain2.mrc"), gain[None], 2, pixelsize_nm=0.5)
    r3 = ImageRegistrator()
    r3.files["gainRef"] = str(tmp_path / "gain2.mrc")
    r3.loadData(str(tmp_path / "movie.mrc"))
    assert r3.pixelsize == np.float32(0.5)
    # 4-bit movie: kept packed
    mo.write(str(tmp_path / "m4.mrc"), raw, 101)
    reg2 = ImageRegistrator()
    reg2.loadData(str(tmp_path / "m4.mrc"))
    assert isinstance(reg2.images, mrc.Packed4) and np.array_equal(mo.unpack4(reg2.images.data, 8), raw)
    with pytest.raises(ValueError, match="3D"):
        mo.write(str(tmp_path / "img.mrc"), raw[:1], 0)
        ImageRegistrator().loadData(str(tmp_path / "img.mrc"))
    with pytest.raises(ValueError, match="not supported"):
        ImageRegistrator().loadData(str(tmp_path / "movie.tif"))


def test_save_data_names_and_contents(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    rng = np.random.default_rng(6)
    reg = ImageRegistrator()
    reg.files["stack"] = "raw/movie_001.mrc"
    reg.pixelsize = np.float32(0.105)
    reg.imageSum = rng.normal(size=(6, 8)).astype(np.float32)
    reg.filtSum = rng.normal(size=(6, 8)).astype(np.float32)
    reg.images = rng.normal(size=(3, 6, 8)).astype(np.float32)
    reg.filterMode = "dose"
    reg.saveData()
    assert reg.files["sum"] == os.path.join("sum", "movie_001_zorro.mrc")
    assert reg.files["align"] == os.path.join("align", "movie_001_zorro_movie.mrcs")
    assert reg.files["filt"] == os.path.join("sum", "movie_001_zorro_filt.mrc")
    s, _, ps = mo.read(reg.files["sum"])
    assert np.array_equal(s[0], reg.imageSum) and abs(ps - 0.105) < 1e-6
    f, _, _ = mo.read(reg.files["filt"])
    assert np.array_equal(f[0], reg.filtSum)
    m, _, _ = mo.read(reg.files["align"])
    assert np.array_equal(m, reg.images)
    reg.files["compressor"] = "zstd"
    with pytest.raises(ValueError, match="compressed"):
        reg.saveData()

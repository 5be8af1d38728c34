"""MRCZ movies (compressed MRC slices, zorro.loadData's .mrcz branch,
zorro.py:3414): LZ4 blocks with known answers, blosc chunks of every layout
the reader takes, MRCZ files through mrc.read and loadData, and the
refusals."""
import struct

import numpy as np
import pytest

from oracle import blosc_oracle
from zorro_gb300 import _lib, blosc, mrc


def _lz4(src, n):
    out = np.zeros(n + 8, dtype=np.uint8)
    s = np.frombuffer(bytes(src), dtype=np.uint8)
    got = _lib.load().zr_lz4_decompress(s.ctypes.data, s.size, out.ctypes.data, n)
    return got, out[:max(got, 0)].tobytes()


def test_lz4_known_answers():
    # literals only (the last sequence of every block)
    assert _lz4(b"\x50hello", 5) == (5, b"hello")
    # 3 literals, an overlapping match of 9 at offset 3, 3 final literals
    assert _lz4(b"\x35abc\x03\x00\x30xyz", 15) == (15, b"abcabcabcabcxyz")
    # a literal length of 15 + 5 in an extra byte
    lits = bytes(range(65, 85))
    assert _lz4(b"\xf0\x05" + lits, 20) == (20, lits)
    # a match length of 15 + 255 + 10 + 4 at offset 1: a run of one byte
    assert _lz4(b"\x1fa\x01\x00\xff\x0a\x10b", 286) == (286, b"a" * 285 + b"b")


@pytest.mark.parametrize("bad", [b"\x35abc\x09\x00", b"\x35abc\x03", b"\xf0", b"\x50hel"])
def test_lz4_malformed_blocks_are_refused(bad):
    got, _ = _lz4(bad, 64)
    assert got == -1


def test_lz4_output_bound_is_enforced():
    got, _ = _lz4(b"\x1fa\x01\x00\xff\x0a\x10b", 100)  # decodes to 286 bytes, 100 allowed
    assert got == -1


@pytest.mark.parametrize("codec", ["zlib", "lz4"])
@pytest.mark.parametrize("typesize,shuffle,split", [(1, False, True), (2, True, True), (2, True, False),
                                                     (4, True, True), (4, False, False)])
def test_blosc_chunks_round_trip(codec, typesize, shuffle, split):
    rng = np.random.default_rng(typesize)
    counts = rng.poisson(0.8, 20000).astype({1: "u1", 2: "<u2", 4: "<f4"}[typesize])
    raw = counts.tobytes() + b"\x07" * 3  # a ragged tail: the last block is short
    ch = blosc_oracle.chunk(raw, typesize, codec, blocksize=8192, shuffle=shuffle, split=split)
    assert blosc.decompress(ch) == raw


def test_blosc_stored_chunk():
    raw = bytes(range(256)) * 3
    assert blosc.decompress(blosc_oracle.chunk(raw, 1, stored=True)) == raw


def test_blosc_refusals():
    raw = bytes(1000)
    ch = bytearray(blosc_oracle.chunk(raw, 4, "zlib", blocksize=512))
    ch[2] |= 0x04  # bit shuffle
    with pytest.raises(blosc.BloscError, match="bit-shuffled"):
        blosc.decompress(bytes(ch))
    ch = bytearray(blosc_oracle.chunk(raw, 4, "zlib", blocksize=512))
    ch[2] = (ch[2] & 0x1f) | (4 << 5)  # zstd
    with pytest.raises(blosc.BloscError, match="zstd"):
        blosc.decompress(bytes(ch))


@pytest.mark.parametrize("mode,compressor", [(0, "zlib"), (6, "lz4"), (12, "lz4hc"), (2, "zlib")])
def test_mrcz_file_reads_like_the_movie(tmp_path, mode, compressor):
    rng = np.random.default_rng(mode)
    movie = rng.poisson(1.2, (3, 40, 50)).astype({0: "u1", 6: "u2", 12: "f2", 2: "f4"}[mode])
    path = str(tmp_path / "movie.mrcz")
    blosc_oracle.write_mrcz(path, movie, mode, compressor, pixelsize_nm=0.105, blocksize=1024)
    data, h = mrc.read(path)
    assert h["compressor"] == compressor and h["mode"] == mode
    assert data.dtype == movie.dtype
    assert np.array_equal(data, movie)
    assert h["pixelsize"][0] == pytest.approx(0.105, rel=1e-6)


def test_load_data_reads_an_mrcz_movie(tmp_path):
    from zorro_gb300.registrator import ImageRegistrator
    movie = np.random.default_rng(9).poisson(1.0, (4, 30, 20)).astype(np.uint8)
    path = str(tmp_path / "m.mrcz")
    blosc_oracle.write_mrcz(path, movie, 0, "zlib", pixelsize_nm=0.05)
    reg = ImageRegistrator()
    reg.loadData(path)
    assert np.array_equal(reg.images, movie)
    assert reg.pixelsize == pytest.approx(0.05, rel=1e-6)


def test_uncompressed_mrcz_is_an_mrc_file(tmp_path):
    from oracle import mrc_oracle
    movie = np.arange(2 * 6 * 5, dtype=np.float32).reshape(2, 6, 5)
    path = str(tmp_path / "plain.mrcz")
    mrc_oracle.write(path, movie, 2)
    data, h = mrc.read(path)
    assert h["compressor"] is None
    assert np.array_equal(data, movie)

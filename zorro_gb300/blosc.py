"""Blosc chunks, the compressed slices of MRCZ movie files (mrcz writes each
z-slice of an MRC stack as one blosc chunk after the header; zorro.loadData
reads .mrcz through mrcz, zorro.py:3414).

A chunk, as the blosc 1 format describes it:

* a 16-byte header: format version, codec format version, flags, the
  element size, then three little-endian uint32: the uncompressed size, the
  block size and the chunk's own size;
* flags: bit 0 byte shuffle, bit 1 stored uncompressed (the data follow the
  header as they are), bit 2 bit shuffle, bit 4 blocks not split, bits 5-7
  the codec (0 blosclz, 1 LZ4 / LZ4HC, 2 snappy, 3 zlib, 4 zstd);
* one little-endian uint32 start offset per block, then the blocks; a block
  is ``splits`` streams (the element size when the block is split: byte
  shuffled or not, element size at most 16, at least 128 elements, not the
  short last block, and bit 4 clear; else one), each a little-endian int32
  compressed size and that many bytes, stored as they are when the size
  equals the stream's uncompressed size;
* a byte-shuffled block holds byte j of every element before byte j + 1.

Decoded here: blocks stored as they are, zlib (Python's zlib) and LZ4 /
LZ4HC (``zr_lz4_decompress``, host code in libzorrogb), unshuffled or
byte-shuffled.  Bit-shuffled chunks and the blosclz, snappy and zstd codecs
are refused by name.
"""
from __future__ import annotations

import ctypes as C
import struct
import zlib

import numpy as np

CODECS = {0: "blosclz", 1: "lz4", 2: "snappy", 3: "zlib", 4: "zstd"}
HEADER = 16


class BloscError(ValueError):
    pass


def chunk_header(buf):
    """(version, codec version, flags, typesize, nbytes, blocksize, cbytes)
    of the chunk at the start of ``buf``."""
    if len(buf) < HEADER:
        raise BloscError("blosc chunk header truncated")
    return struct.unpack("<BBBBIII", bytes(buf[:HEADER]))


def _lz4(src, n):
    from . import _lib
    out = np.empty(n, dtype=np.uint8)
    s = np.frombuffer(src, dtype=np.uint8)
    got = _lib.load().zr_lz4_decompress(s.ctypes.data_as(C.c_void_p), s.size, out.ctypes.data_as(C.c_void_p), n)
    if got != n:
        raise BloscError("LZ4 stream decodes to %d bytes, not %d" % (got, n))
    return out.tobytes()


def _stream(codec, src, n):
    if len(src) == n:  # stored as it is
        return bytes(src)
    if codec == 3:
        out = zlib.decompress(bytes(src))
    elif codec == 1:
        out = _lz4(bytes(src), n)
    else:
        raise BloscError("blosc codec %s is not supported (zlib and LZ4/LZ4HC are)" % CODECS.get(codec, codec))
    if len(out) != n:
        raise BloscError("blosc stream decodes to %d bytes, not %d" % (len(out), n))
    return out


def decompress(chunk):
    """The uncompressed bytes of one blosc chunk."""
    ver, verlz, flags, typesize, nbytes, blocksize, cbytes = chunk_header(chunk)
    if cbytes > len(chunk):
        raise BloscError("blosc chunk truncated: %d of %d bytes" % (len(chunk), cbytes))
    if flags & 0x04:
        raise BloscError("bit-shuffled blosc chunks are not supported (byte shuffle and none are)")
    if flags & 0x02:  # stored uncompressed
        if HEADER + nbytes > cbytes:
            raise BloscError("blosc chunk shorter than its stored data")
        return bytes(chunk[HEADER:HEADER + nbytes])
    codec = (flags >> 5) & 0x7
    shuffle = bool(flags & 0x01) and typesize > 1
    dont_split = bool(flags & 0x10)
    if blocksize <= 0:
        raise BloscError("blosc block size %d" % blocksize)
    nblocks = (nbytes + blocksize - 1) // blocksize
    starts = struct.unpack("<%dI" % nblocks, bytes(chunk[HEADER:HEADER + 4 * nblocks]))
    out = bytearray(nbytes)
    for j, start in enumerate(starts):
        bsize = min(blocksize, nbytes - j * blocksize)
        leftover = bsize < blocksize
        splits = typesize if (not dont_split and typesize <= 16 and bsize // typesize >= 128 and not leftover) else 1
        neblock = bsize // splits
        pos = start
        parts = []
        for _ in range(splits):
            (csize,) = struct.unpack("<i", bytes(chunk[pos:pos + 4]))
            pos += 4
            if csize < 0 or pos + csize > cbytes:
                raise BloscError("blosc stream of %d bytes overruns the chunk" % csize)
            parts.append(_stream(codec, chunk[pos:pos + csize], neblock))
            pos += csize
        block = b"".join(parts)
        if shuffle:
            n = bsize // typesize
            body = np.frombuffer(block[:n * typesize], dtype=np.uint8).reshape(typesize, n).T.tobytes()
            block = body + block[n * typesize:]
        out[j * blocksize:j * blocksize + bsize] = block
    return bytes(out)

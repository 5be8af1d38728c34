"""Blosc chunks and MRCZ files written from the formats' descriptions, for
the reader's tests.

TEST INFRASTRUCTURE ONLY: only ``tests/`` uses it.  ``lz4_block`` is a small
greedy LZ4 block encoder (literal runs and matches, the match search limited
to runs of one repeated byte and to the previous sequence's literals, enough
to produce long literal and match lengths and overlapping matches);
``chunk`` lays out a blosc 1 chunk (header, block starts, split streams,
byte shuffle, zlib or LZ4 streams, or stored data); ``write_mrcz`` writes an
MRC file with the compressor code in the mode word's thousands and one
chunk per z-slice.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

from oracle import mrc_oracle

CODEC_FLAGS = {"lz4": 1, "zlib": 3}
MRCZ_CODES = {"lz4": 2, "lz4hc": 3, "zlib": 5}


def _length_bytes(n):
    out = b""
    while n >= 255:
        out += b"\xff"
        n -= 255
    return out + bytes([n])


def lz4_block(data):
    """An LZ4 block of ``data``: greedy matches of repeated-byte runs
    (offset 1) of at least 4 bytes, literals elsewhere, and a final
    literal-only sequence of the last bytes."""
    data = bytes(data)
    n = len(data)
    out = bytearray()
    lit_start = 0
    i = 1
    while i < n - 5:
        run = 0
        while i + run < n - 5 and data[i + run] == data[i - 1]:
            run += 1
        if run >= 4:
            lit = data[lit_start:i]
            mlen = run - 4
            out.append((min(len(lit), 15) << 4) | min(mlen, 15))
            if len(lit) >= 15:
                out += _length_bytes(len(lit) - 15)
            out += lit
            out += struct.pack("<H", 1)
            if mlen >= 15:
                out += _length_bytes(mlen - 15)
            i += run
            lit_start = i
            i += 1
        else:
            i += 1
    lit = data[lit_start:]
    out.append(min(len(lit), 15) << 4)
    if len(lit) >= 15:
        out += _length_bytes(len(lit) - 15)
    out += lit
    return bytes(out)


def _encode(codec, data):
    if codec == "zlib":
        return zlib.compress(data, 6)
    return lz4_block(data)


def chunk(data, typesize, codec="zlib", blocksize=4096, shuffle=True, split=True, stored=False):
    """A blosc 1 chunk of ``data`` (bytes)."""
    data = bytes(data)
    nbytes = len(data)
    flags = (0x01 if shuffle else 0) | (0x02 if stored else 0) | (0x00 if split else 0x10)
    flags |= CODEC_FLAGS[codec] << 5
    if stored:
        cbytes = 16 + nbytes
        return struct.pack("<BBBBIII", 2, 1, flags, typesize, nbytes, blocksize, cbytes) + data
    nblocks = (nbytes + blocksize - 1) // blocksize
    blocks = []
    for j in range(nblocks):
        blk = data[j * blocksize:(j + 1) * blocksize]
        bsize = len(blk)
        if shuffle and typesize > 1:
            n = bsize // typesize
            body = np.frombuffer(blk[:n * typesize], dtype=np.uint8).reshape(n, typesize).T.tobytes()
            blk = body + blk[n * typesize:]
        leftover = bsize < blocksize
        splits = typesize if (split and typesize <= 16 and bsize // typesize >= 128 and not leftover) else 1
        neb = bsize // splits
        out = b""
        for k in range(splits):
            part = blk[k * neb:(k + 1) * neb]
            enc = _encode(codec, part)
            if len(enc) >= len(part):
                enc = part  # stored as it is
            out += struct.pack("<i", len(enc)) + enc
        blocks.append(out)
    starts = []
    pos = 16 + 4 * nblocks
    for b in blocks:
        starts.append(pos)
        pos += len(b)
    head = struct.pack("<BBBBIII", 2, 1, flags, typesize, nbytes, blocksize, pos)
    return head + struct.pack("<%dI" % nblocks, *starts) + b"".join(blocks)


def write_mrcz(path, data, mode, compressor="zlib", pixelsize_nm=1.0, **chunk_kw):
    """An MRCZ file: the MRC header with mode + 1000 x the compressor's code,
    then one blosc chunk per z-slice."""
    a = np.asarray(data)
    mrc_oracle.write(path, a[:1], mode, pixelsize_nm)
    with open(path, "r+b") as fh:
        head = bytearray(fh.read(1024))
    struct.pack_into("<3i", head, 0, a.shape[2], a.shape[1], a.shape[0])
    struct.pack_into("<i", head, 12, mode + 1000 * MRCZ_CODES[compressor])
    struct.pack_into("<3i", head, 28, a.shape[2], a.shape[1], a.shape[0])
    struct.pack_into("<3f", head, 40, 10.0 * pixelsize_nm * a.shape[2], 10.0 * pixelsize_nm * a.shape[1],
                     10.0 * pixelsize_nm * a.shape[0])
    dt = {0: "u1", 1: "<i2", 2: "<f4", 6: "<u2", 12: "<f2"}[mode]
    codec = "lz4" if compressor in ("lz4", "lz4hc") else compressor
    with open(path, "wb") as fh:
        fh.write(bytes(head))
        for z in range(a.shape[0]):
            sl = a[z].astype(dt)
            fh.write(chunk(sl.tobytes(), sl.dtype.itemsize, codec, **chunk_kw))
    return path

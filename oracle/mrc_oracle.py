"""CPU restatement of the MRC movie format the reference reads and writes.

TEST INFRASTRUCTURE ONLY: the checker for ``zorro_gb300.mrc`` and for the GPU
4-bit unpack (``zr_unpack_u4``); the product never calls it.

The reference reads movies with mrcz.readMRC (zorro/zorro.py:3414-3425;
mrcz >= 0.0.1, requirements.txt:5, not installed here) and writes sums with
mrcz.writeMRC (zorro.py:3583, 3603, 3621).  mrcz implements the published
MRC2014 layout with the IMOD conventions; this module restates that layout
from the format description with a NumPy structured header, independently
of the product's struct-based parser:

  header  1024 bytes: words 0-2 nx, ny, nz; 3 mode; 7-9 mx, my, mz; 10-12
          cell lengths (Angstrom); 23 extended-header bytes; bytes 152-159 the
          IMOD stamp (1146047817) and flags (bit 1: bytes are signed); 208
          "MAP "; 212 machine stamp (0x44 0x44: little-endian, 0x11 0x11: big)
  data    after the extended header, x fastest
  modes   0 bytes (unsigned with the IMOD stamp and no signed flag), 1 int16,
          2 float32, 4 complex64, 6 uint16, 12 float16, 101 two 4-bit pixels a
          byte, the first in the low nibble, rows padded to whole bytes

Parity: no mrcz output exists in the reference tree, so the format is pinned
by known-answer cases written from the description (see tests/test_mrc.py).
"""
from __future__ import annotations

import numpy as np

_HDR = [("nx", "i4"), ("ny", "i4"), ("nz", "i4"), ("mode", "i4"), ("start", "i4", 3), ("m", "i4", 3),
        ("cella", "f4", 3), ("cellb", "f4", 3), ("mapcrs", "i4", 3), ("dmin", "f4"), ("dmax", "f4"),
        ("dmean", "f4"), ("ispg", "i4"), ("nsymbt", "i4"), ("extra1", "V8"), ("exttyp", "S4"),
        ("nversion", "i4"), ("extra2", "V40"), ("imod_stamp", "i4"), ("imod_flags", "i4"), ("extra3", "V36"),
        ("origin", "f4", 3), ("map", "S4"), ("machst", "V4"), ("rms", "f4"), ("nlabl", "i4"),
        ("labels", "S80", 10)]


def header_dtype(order="<"):
    dt = np.dtype([(f[0], order + f[1] if f[1][0] in "if" else f[1]) + tuple(f[2:]) for f in _HDR])
    assert dt.itemsize == 1024
    return dt


def read_header(raw):
    st = bytes(raw[212:214])
    order = ">" if st == b"\x11\x11" else "<"
    return np.frombuffer(bytes(raw[:1024]), dtype=header_dtype(order))[0], order


def unpack4(packed, nx):
    """[..., (nx+1)//2] bytes -> [..., nx] uint8 pixels, low nibble first."""
    p = np.asarray(packed, dtype=np.uint8)
    both = np.stack([p & 0x0F, p >> 4], axis=-1).reshape(p.shape[:-1] + (2 * p.shape[-1],))
    return np.ascontiguousarray(both[..., :nx])


def pack4(pixels):
    """[..., nx] values 0..15 -> [..., (nx+1)//2] bytes (odd rows padded)."""
    a = np.asarray(pixels, dtype=np.uint8)
    if a.shape[-1] % 2:
        a = np.concatenate([a, np.zeros(a.shape[:-1] + (1,), np.uint8)], axis=-1)
    return np.ascontiguousarray(a[..., 0::2] | (a[..., 1::2] << 4))


def read(path):
    """(pixels [nz][ny][nx], header record, pixel size in nm along x)."""
    raw = open(path, "rb").read()
    h, order = read_header(raw)
    nx, ny, nz, mode = int(h["nx"]), int(h["ny"]), int(h["nz"]), int(h["mode"])
    off = 1024 + int(h["nsymbt"])
    if mode == 101:
        rb = (nx + 1) // 2
        packed = np.frombuffer(raw, dtype=np.uint8, count=nz * ny * rb, offset=off).reshape(nz, ny, rb)
        data = unpack4(packed, nx)
    else:
        if mode == 0:
            unsigned = int(h["imod_stamp"]) == 1146047817 and not (int(h["imod_flags"]) & 1)
            dt = np.dtype("u1" if unsigned else "i1")
        else:
            dt = np.dtype(order + {1: "i2", 2: "f4", 4: "c8", 6: "u2", 12: "f2"}[mode])
        data = np.frombuffer(raw, dtype=dt, count=nz * ny * nx, offset=off).reshape(nz, ny, nx).astype(
            dt.newbyteorder("="))
    mx = int(h["m"][0])
    ps = float(h["cella"][0]) / mx / 10.0 if mx > 0 else 0.0
    return data, h, ps


def write(path, data, mode, pixelsize_nm=1.0, order="<", signed_bytes=False, imod=True, nsymbt=0):
    """An MRC file of ``data`` in ``mode`` (101: ``data`` are 4-bit pixel
    values), written with a structured header in byte order ``order``."""
    a = np.asarray(data)
    nz, ny, nx = a.shape
    h = np.zeros((), dtype=header_dtype(order))
    h["nx"], h["ny"], h["nz"], h["mode"] = nx, ny, nz, mode
    h["m"] = (nx, ny, nz)
    h["cella"] = (10.0 * pixelsize_nm * nx, 10.0 * pixelsize_nm * ny, 10.0 * pixelsize_nm * nz)
    h["cellb"] = (90.0, 90.0, 90.0)
    h["mapcrs"] = (1, 2, 3)
    h["nsymbt"] = nsymbt
    if imod:
        h["imod_stamp"] = 1146047817
        h["imod_flags"] = 1 if signed_bytes else 0
    h["map"] = b"MAP "
    h["machst"] = np.frombuffer(b"\x11\x11\x00\x00" if order == ">" else b"\x44\x44\x00\x00", dtype="V4")[0]
    if mode == 101:
        body = pack4(a).tobytes()
    else:
        dt = {0: "i1" if signed_bytes else "u1", 1: "i2", 2: "f4", 4: "c8", 6: "u2", 12: "f2"}[mode]
        dt = np.dtype(dt if dt[-1] == "1" else order + dt)
        body = a.astype(dt).tobytes()
    with open(path, "wb") as fh:
        fh.write(h.tobytes())
        fh.write(b"\x00" * nsymbt)
        fh.write(body)
    return path

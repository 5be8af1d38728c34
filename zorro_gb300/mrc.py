"""MRC files: the movie, sum and gain-reference format of zorro.loadData /
saveData (zorro.py:3414-3425, 3573-3627), which the reference reads and
writes through mrcz (requirements.txt:5, mrcz >= 0.0.1, not bundled).

The layout follows the MRC2014 standard with the IMOD extensions the
detector software writes:

* a 1024-byte header of 4-byte words (little- or big-endian, told by the
  machine stamp at byte 212), followed by ``nsymbt`` bytes of extended
  header, then the data, x fastest: a stack reads as [nz][ny][nx];
* data modes 0 (bytes), 1 (int16), 2 (float32), 4 (complex64), 6 (uint16),
  12 (float16) and 101 (4-bit pixels, two per byte, the first in the low four
  bits, each row padded to a whole byte);
* mode-0 bytes are unsigned when the IMOD stamp is present without its
  "signed bytes" flag (imodFlags bit 1), signed otherwise;
* the pixel size is the cell length over the sampling (cella.x / mx, in
  Angstrom); the registrator keeps it in nm, as mrcz's pixelunits='nm' does.

``read(..., pinned=True)`` reads the data block straight into page-locked
host memory, so the copy to the GPU is one asynchronous transfer.  A mode-101
movie is returned packed (``Packed4``): the packed bytes are what crosses the
host link, and the GPU path expands them in HBM (``zr_unpack_u4``).

MRCZ files are MRC files whose mode word also names a compressor (mode +
1000 x code: 1 blosclz, 2 lz4, 3 lz4hc, 4 snappy, 5 zlib, 6 zstd) and whose
z-slices follow the header as one blosc chunk each (``blosc``); without a
compressor an .mrcz file is a plain MRC file.  .bz2/.gz files are not read.
"""
from __future__ import annotations

import os
import struct

import numpy as np

HEADER_BYTES = 1024
IMOD_STAMP = 1146047817
IMOD_SIGNED_BYTES = 1
MODE_U4 = 101
MRCZ_COMPRESSORS = {0: None, 1: "blosclz", 2: "lz4", 3: "lz4hc", 4: "snappy", 5: "zlib", 6: "zstd"}
_MODE_DTYPES = {1: "i2", 2: "f4", 4: "c8", 6: "u2", 12: "f2"}
_DTYPE_MODES = {"int8": 0, "uint8": 0, "int16": 1, "float32": 2, "complex64": 4, "uint16": 6, "float16": 12}


class Packed4:
    """A 4-bit (mode 101) stack as stored: ``data`` is uint8
    [nz][ny][(nx + 1) // 2], two pixels a byte, the first in the low four
    bits; ``shape`` is the pixel shape (nz, ny, nx)."""

    def __init__(self, data, shape):
        self.data = data
        self.shape = tuple(int(v) for v in shape)
        if self.data.shape != (self.shape[0], self.shape[1], (self.shape[2] + 1) // 2):
            raise ValueError("packed 4-bit data %s does not match pixel shape %s" % (self.data.shape, self.shape))

    ndim = 3
    dtype = "uint4"

    @property
    def nbytes(self):
        return self.data.nbytes

    def __len__(self):
        return self.shape[0]


def _byteorder(raw):
    stamp = raw[212:214]
    if stamp in (b"\x44\x44", b"\x44\x41"):
        return "<"
    if stamp == b"\x11\x11":
        return ">"
    # no stamp (older writers): the order in which the mode word is sane
    for bo in ("<", ">"):
        mode = struct.unpack(bo + "i", raw[12:16])[0]
        if mode >= 0 and mode % 1000 in (0, 1, 2, 4, 6, 12, MODE_U4) and mode // 1000 in MRCZ_COMPRESSORS:
            return bo
    raise ValueError("not an MRC file: unknown byte order and mode")


def parse_header(raw):
    """The fields of a 1024-byte MRC header (bytes) as a dict."""
    if len(raw) < HEADER_BYTES:
        raise ValueError("MRC header truncated (%d bytes)" % len(raw))
    bo = _byteorder(raw)
    w = struct.unpack(bo + "10i6f3i3f2i", raw[:96])
    h = {"nx": w[0], "ny": w[1], "nz": w[2], "mode": w[3], "nxstart": w[4], "nystart": w[5], "nzstart": w[6],
         "mx": w[7], "my": w[8], "mz": w[9], "cella": w[10:13], "cellb": w[13:16], "mapc": w[16], "mapr": w[17],
         "maps": w[18], "dmin": w[19], "dmax": w[20], "dmean": w[21], "ispg": w[22], "nsymbt": w[23]}
    h["exttyp"] = raw[104:108]
    h["nversion"] = struct.unpack(bo + "i", raw[108:112])[0]
    h["imodStamp"], h["imodFlags"] = struct.unpack(bo + "2i", raw[152:160])
    h["origin"] = struct.unpack(bo + "3f", raw[196:208])
    h["map"] = raw[208:212]
    h["rms"] = struct.unpack(bo + "f", raw[216:220])[0]
    nl = struct.unpack(bo + "i", raw[220:224])[0]
    h["labels"] = [raw[224 + 80 * i:304 + 80 * i].rstrip(b"\x00 ").decode("latin-1") for i in range(max(0, min(nl, 10)))]
    h["byteorder"] = bo
    # MRCZ: the compressor in the thousands of the mode word
    if h["mode"] >= 1000:
        if h["mode"] // 1000 not in MRCZ_COMPRESSORS:
            raise ValueError("MRC mode %d: unknown compressor code %d" % (h["mode"], h["mode"] // 1000))
        h["compressor"] = MRCZ_COMPRESSORS[h["mode"] // 1000]
        h["mode"] %= 1000
    else:
        h["compressor"] = None
    if h["nx"] <= 0 or h["ny"] <= 0 or h["nz"] <= 0:
        raise ValueError("MRC header with empty shape %s" % ((h["nx"], h["ny"], h["nz"]),))
    # Angstrom per pixel along x, y, z (0 where the sampling is unset)
    h["pixelsize_A"] = tuple(float(c) / m if m > 0 else 0.0 for c, m in zip(h["cella"], (h["mx"], h["my"], h["mz"])))
    h["pixelsize"] = tuple(v / 10.0 for v in h["pixelsize_A"])  # nm
    return h


def data_dtype(h):
    """NumPy dtype of the data block (None for mode 101)."""
    mode = h["mode"]
    if mode == MODE_U4:
        return None
    if mode == 0:
        signed = not (h["imodStamp"] == IMOD_STAMP and not (h["imodFlags"] & IMOD_SIGNED_BYTES))
        return np.dtype("i1" if signed else "u1")
    if mode not in _MODE_DTYPES:
        raise ValueError("MRC mode %d not supported" % mode)
    return np.dtype(h["byteorder"] + _MODE_DTYPES[mode])


def read_header(path):
    with open(path, "rb") as fh:
        return parse_header(fh.read(HEADER_BYTES))


def _host_buffer(nbytes, pinned):
    """Host memory for the data block: page-locked when asked for and a CUDA
    device exists (pinning only speeds up the later device copy)."""
    if pinned:
        import torch
        if torch.cuda.is_available():
            return torch.empty(nbytes, dtype=torch.uint8, pin_memory=True).numpy()
    return np.empty(nbytes, dtype=np.uint8)


def read(path, pinned=False):
    """(data, header) of an MRC file.  ``data`` is [nz][ny][nx] in the file's
    own type (native byte order), or a ``Packed4`` for mode 101.  With
    ``pinned`` the data live in page-locked host memory."""
    ext = os.path.splitext(str(path))[1].lower()
    if ext in (".bz2", ".gz", ".7z"):
        raise ValueError("compressed files (%s) are not read: decompress first" % ext)
    with open(path, "rb") as fh:
        h = parse_header(fh.read(HEADER_BYTES))
        fh.seek(HEADER_BYTES + max(0, h["nsymbt"]))
        nz, ny, nx = h["nz"], h["ny"], h["nx"]
        dt = data_dtype(h)
        slice_bytes = ny * ((nx + 1) // 2) if dt is None else ny * nx * dt.itemsize
        nbytes = nz * slice_bytes
        buf = _host_buffer(nbytes, pinned)
        if h["compressor"] is None:
            got = fh.readinto(memoryview(buf))
        else:
            got = _read_blosc_slices(fh, nz, slice_bytes, buf)
    if got != nbytes:
        raise ValueError("MRC data truncated: %d of %d bytes" % (got, nbytes))
    if dt is None:
        return Packed4(buf.reshape(nz, ny, (nx + 1) // 2), (nz, ny, nx)), h
    a = buf.view(dt).reshape(nz, ny, nx)
    if dt.byteorder == ">":
        a = a.byteswap(inplace=True).view(dt.newbyteorder("="))
    return a, h


def _read_blosc_slices(fh, nz, slice_bytes, buf):
    """MRCZ data: one blosc chunk per z-slice, each as long as its header
    says; decoded into ``buf``.  Returns the bytes decoded."""
    from . import blosc
    got = 0
    for z in range(nz):
        head = fh.read(blosc.HEADER)
        if len(head) < blosc.HEADER:
            break
        cbytes = blosc.chunk_header(head)[6]
        chunk = head + fh.read(cbytes - blosc.HEADER)
        data = blosc.decompress(chunk)
        if len(data) != slice_bytes:
            raise ValueError("MRCZ slice %d holds %d bytes, not %d" % (z, len(data), slice_bytes))
        buf[z * slice_bytes:(z + 1) * slice_bytes] = np.frombuffer(data, dtype=np.uint8)
        got += len(data)
    return got


def _stats(a):
    if a.size == 0 or np.iscomplexobj(a):
        return 0.0, 0.0, 0.0, -1.0
    a64 = a.astype(np.float64, copy=False)
    return float(a64.min()), float(a64.max()), float(a64.mean()), float(a64.std())


def write(path, data, pixelsize=None, label="zorro_gb300"):
    """Write ``data`` ([nz][ny][nx] or [ny][nx] array, or a Packed4) as a
    little-endian MRC2014 file.  ``pixelsize`` in nm (a number, or per axis
    (x, y, z)); unset leaves the cell equal to the pixel counts x 1 A."""
    if isinstance(data, Packed4):
        body, (nz, ny, nx), mode, flags = np.ascontiguousarray(data.data), data.shape, MODE_U4, 0
        dmin, dmax, dmean, rms = 0.0, 15.0, 0.0, -1.0
    else:
        a = np.asarray(data)
        if a.ndim == 2:
            a = a[None]
        if a.ndim != 3:
            raise ValueError("MRC data must be 2-D or 3-D, not %d-D" % a.ndim)
        if a.dtype == np.float64:
            a = a.astype(np.float32)
        if a.dtype.name not in _DTYPE_MODES:
            raise ValueError("no MRC mode for dtype %s" % a.dtype)
        body = np.ascontiguousarray(a, dtype=a.dtype.newbyteorder("<"))
        nz, ny, nx = a.shape
        mode = _DTYPE_MODES[a.dtype.name]
        flags = IMOD_SIGNED_BYTES if a.dtype == np.int8 else 0
        dmin, dmax, dmean, rms = _stats(a)
    if pixelsize is None:
        ps = (1.0, 1.0, 1.0)
    elif np.ndim(pixelsize) == 0:
        ps = (10.0 * float(pixelsize),) * 3
    else:
        p = [10.0 * float(v) for v in pixelsize]
        ps = tuple(p + [p[-1]] * (3 - len(p)))
    hdr = bytearray(HEADER_BYTES)
    struct.pack_into("<10i6f3i3f2i", hdr, 0, nx, ny, nz, mode, 0, 0, 0, nx, ny, nz,
                     ps[0] * nx, ps[1] * ny, ps[2] * nz, 90.0, 90.0, 90.0, 1, 2, 3, dmin, dmax, dmean, 0, 0)
    hdr[104:108] = b"\x00\x00\x00\x00"
    struct.pack_into("<i", hdr, 108, 20140)
    struct.pack_into("<2i", hdr, 152, IMOD_STAMP, flags)
    hdr[208:212] = b"MAP "
    hdr[212:216] = b"\x44\x44\x00\x00"
    struct.pack_into("<f", hdr, 216, rms)
    lab = label.encode("latin-1")[:80] if label else b""
    struct.pack_into("<i", hdr, 220, 1 if lab else 0)
    hdr[224:224 + len(lab)] = lab
    d = os.path.dirname(os.path.abspath(str(path)))
    os.makedirs(d, exist_ok=True)
    with open(path, "wb") as fh:
        fh.write(bytes(hdr))
        fh.write(memoryview(body.reshape(-1).view(np.uint8)))
    return path

"""DigitalMicrograph 4 (.dm4) movies: the DM4 branch of zorro.loadData
(zorro.py:3384-3411), which the reference reads through mrcz.readDM4 (not
bundled with it).

A DM4 file is a tree of tags, laid out as the format's published
description gives it:

* file header, big-endian: version (uint32, 4), length of the root
  directory (uint64), byte order of the tag data (uint32: 1 little-endian,
  0 big-endian);
* a tag directory: sorted (uint8), open (uint8), number of tags (uint64),
  then the tags;
* a tag: kind (uint8: 20 directory, 21 data), name length (uint16, big-endian),
  name, total length of the rest (uint64); a directory tag continues as a
  directory, a data tag with the marker ``%%%%``, the number of info words
  (uint64) and the info words (uint64 each, big-endian), then its value in
  the file's byte order;
* info words: one type code for a number (2 int16, 3 int32, 4 uint16,
  5 uint32, 6 float32, 7 float64, 8 bool, 9 int8, 10 uint8, 11 int64,
  12 uint64); ``18, n`` for a string of n UTF-16 code units; ``15, name
  length, n fields, (name length, type) x n`` for a struct; ``20, type, n``
  for an array of n numbers, ``20, 15, ..., n`` for an array of structs.

The images are the groups of ``ImageList``; the first is usually the
thumbnail, and zorro takes the second (``dm4obj.im[1]``).  An image's
``ImageData`` holds ``Data`` (the pixels, x fastest), ``DataType``,
``Dimensions`` (x, y[, z]) and ``Calibrations/Dimension`` (per axis
``Scale`` and ``Units``; DigitalMicrograph writes nm).  ``ImageTags`` holds
the microscope's settings (``Microscope Info/Voltage`` in V,
``Microscope Info/Cs(mm)``).
"""
from __future__ import annotations

import struct

import numpy as np

# data tag type codes -> (struct code, numpy dtype)
_TYPES = {2: ("h", "i2"), 3: ("i", "i4"), 4: ("H", "u2"), 5: ("I", "u4"), 6: ("f", "f4"), 7: ("d", "f8"),
          8: ("?", "u1"), 9: ("b", "i1"), 10: ("B", "u1"), 11: ("q", "i8"), 12: ("Q", "u8")}
# ImageData/DataType -> numpy dtype of the pixels
_IMAGE_TYPES = {1: "i2", 2: "f4", 3: "c8", 6: "u1", 7: "i4", 9: "i1", 10: "u2", 11: "u4", 12: "f8", 13: "c16"}


class DM4Error(ValueError):
    pass


class _Reader:
    def __init__(self, buf):
        self.buf = buf
        self.pos = 0

    def take(self, n):
        if self.pos + n > len(self.buf):
            raise DM4Error("DM4 file truncated at byte %d" % self.pos)
        b = self.buf[self.pos:self.pos + n]
        self.pos += n
        return b

    def be(self, fmt):
        size = struct.calcsize(">" + fmt)
        return struct.unpack(">" + fmt, self.take(size))[0]


def _value(r, info, bo):
    """The value of a data tag from its info words (``bo``: '<' or '>')."""
    kind = info[0]
    if kind in _TYPES:
        code, _ = _TYPES[kind]
        return struct.unpack(bo + code, r.take(struct.calcsize(code)))[0]
    if kind == 18:  # string of UTF-16 code units
        n = info[1]
        return bytes(r.take(2 * n)).decode("utf-16-le" if bo == "<" else "utf-16-be", errors="replace")
    if kind == 15:  # struct: fields after (name length, n fields), two words each
        nf = info[2]
        return tuple(_value(r, [info[4 + 2 * k]], bo) for k in range(nf))
    if kind == 20:
        elem = info[1]
        if elem == 15:  # array of structs
            nf = info[3]
            types = [info[5 + 2 * k] for k in range(nf)]
            count = info[4 + 2 * nf]
            return [tuple(_value(r, [t], bo) for t in types) for _ in range(count)]
        if elem not in _TYPES:
            raise DM4Error("DM4 array of type %d not supported" % elem)
        count = info[2]
        _, dt = _TYPES[elem]
        raw = r.take(count * np.dtype(dt).itemsize)
        return np.frombuffer(raw, dtype=np.dtype(dt).newbyteorder(bo))
    raise DM4Error("DM4 tag type %d not supported" % kind)


def _directory(r, bo):
    """A tag directory as a list of (name, value) in file order; a nested
    directory's value is such a list itself."""
    r.take(2)  # sorted, open
    n = r.be("Q")
    out = []
    for _ in range(n):
        kind = r.be("B")
        if kind == 0:  # end of file
            break
        name = bytes(r.take(r.be("H"))).decode("latin-1")
        length = r.be("Q")
        end = r.pos + length
        if kind == 20:
            out.append((name, _directory(r, bo)))
        elif kind == 21:
            if bytes(r.take(4)) != b"%%%%":
                raise DM4Error("DM4 data tag %r without its %%%%%% marker" % name)
            ninfo = r.be("Q")
            info = [r.be("Q") for _ in range(ninfo)]
            out.append((name, _value(r, info, bo)))
        else:
            raise DM4Error("DM4 tag kind %d at byte %d" % (kind, r.pos))
        if length and r.pos != end:
            r.pos = end  # the declared length rules (padding, unknown fields)
    return out


def parse(buf):
    """The tag tree of a DM4 file (bytes): (byte order, root directory)."""
    r = _Reader(memoryview(buf))
    version = r.be("I")
    if version != 4:
        raise DM4Error("not a DM4 file (version %d)" % version)
    r.be("Q")  # root length
    bo = "<" if r.be("I") == 1 else ">"
    return bo, _directory(r, bo)


def _get(d, path):
    """Value at a '/'-separated path of names in a directory list (None when
    absent)."""
    for name in path.split("/"):
        if not isinstance(d, list):
            return None
        hit = [v for k, v in d if k == name]
        if not hit:
            return None
        d = hit[0]
    return d


def images(tree):
    """The ImageList entries: dicts of ``data`` ([z][y][x] or [y][x]),
    ``scale`` (x axis, as written), ``units``, ``voltage`` (V) and ``cs``
    (mm) when present."""
    bo, root = tree
    out = []
    for _, img in (_get(root, "ImageList") or []):
        dtype = _IMAGE_TYPES.get(int(_get(img, "ImageData/DataType") or 0))
        data = _get(img, "ImageData/Data")
        dims = [int(v) for _, v in (_get(img, "ImageData/Dimensions") or [])]
        if dtype is None or data is None or not dims:
            continue
        # the pixels whatever element type the Data array was written with,
        # in the file's byte order
        pix = np.frombuffer(np.ascontiguousarray(data).tobytes(), dtype=np.dtype(dtype).newbyteorder(bo))
        if pix.size != int(np.prod(dims)):
            raise DM4Error("DM4 image data of %d pixels for dimensions %s" % (pix.size, dims))
        pix = pix.astype(np.dtype(dtype).newbyteorder("="), copy=False).reshape(dims[::-1])
        cal = _get(img, "ImageData/Calibrations/Dimension") or []
        scale = units = None
        if cal:
            scale = _get(cal[0][1], "Scale")
            units = _get(cal[0][1], "Units")
            if isinstance(units, np.ndarray):  # UTF-16 code units
                units = "".join(chr(int(c)) for c in units)
        out.append({"data": pix, "scale": None if scale is None else float(scale), "units": units,
                    "voltage": _get(img, "ImageTags/Microscope Info/Voltage"),
                    "cs": _get(img, "ImageTags/Microscope Info/Cs(mm)")})
    return out


def read(path):
    """(frames, info) of a DM4 movie: the image zorro takes (the second of
    the ImageList, the first being the thumbnail; the only one otherwise)
    and its ``pixelsize`` (nm, None without units), ``voltage`` (kV) and
    ``C3`` (mm) as zorro.loadData sets them (zorro.py:3386-3410)."""
    with open(path, "rb") as fh:
        buf = fh.read()
    ims = images(parse(buf))
    if not ims:
        raise DM4Error("%s holds no image" % path)
    im = ims[1] if len(ims) > 1 else ims[0]
    info = {"pixelsize": None, "voltage": None, "C3": None}
    if im["scale"] and im["units"] not in (None, "", "\x14\x00"):
        info["pixelsize"] = im["scale"]  # DigitalMicrograph calibrates in nm
    if im["voltage"]:
        info["voltage"] = float(im["voltage"]) / 1000.0
    if im["cs"]:
        info["C3"] = float(im["cs"])
    return im["data"], info

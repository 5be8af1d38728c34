"""An independent DM4 writer, for the reader's tests.

TEST INFRASTRUCTURE ONLY: only ``tests/`` uses it.  It writes the
DigitalMicrograph 4 tag-file layout as the format's published description
gives it (big-endian file header and tag framing, 8-byte lengths and info
words, tag values in the declared byte order), so that
``zorro_gb300.dm4`` can be checked on files it did not write itself.
"""
from __future__ import annotations

import struct

import numpy as np

_CODES = {np.dtype("i2"): 2, np.dtype("i4"): 3, np.dtype("u2"): 4, np.dtype("u4"): 5, np.dtype("f4"): 6,
          np.dtype("f8"): 7, np.dtype("i1"): 9, np.dtype("u1"): 10, np.dtype("i8"): 11, np.dtype("u8"): 12}
IMAGE_TYPES = {np.dtype("i2"): 1, np.dtype("f4"): 2, np.dtype("u1"): 6, np.dtype("i4"): 7, np.dtype("i1"): 9,
               np.dtype("u2"): 10, np.dtype("u4"): 11, np.dtype("f8"): 12}


def _data_tag(name, value, bo):
    if isinstance(value, bool):
        info, payload = [8], struct.pack(bo + "?", value)
    elif isinstance(value, int):
        info, payload = [3], struct.pack(bo + "i", value)
    elif isinstance(value, float):
        info, payload = [7], struct.pack(bo + "d", value)
    elif isinstance(value, str):  # as DigitalMicrograph writes text: uint16 code units
        a = np.array([ord(c) for c in value], dtype=np.dtype("u2").newbyteorder(bo))
        info, payload = [20, 4, len(value)], a.tobytes()
    else:
        a = np.asarray(value)
        code = _CODES[a.dtype.newbyteorder("=")]
        info, payload = [20, code, a.size], a.astype(a.dtype.newbyteorder(bo)).tobytes()
    body = b"%%%%" + struct.pack(">Q", len(info)) + b"".join(struct.pack(">Q", v) for v in info) + payload
    nm = name.encode("latin-1")
    return struct.pack(">BH", 21, len(nm)) + nm + struct.pack(">Q", len(body)) + body


def _dir_body(entries, bo):
    tags = b"".join(_tag(k, v, bo) for k, v in entries)
    return struct.pack(">BBQ", 0, 1, len(entries)) + tags


def _tag(name, value, bo):
    if isinstance(value, list):
        body = _dir_body(value, bo)
        nm = name.encode("latin-1")
        return struct.pack(">BH", 20, len(nm)) + nm + struct.pack(">Q", len(body)) + body
    return _data_tag(name, value, bo)


def dm4_bytes(images, little_endian=True):
    """A DM4 file holding ``images``: a list of dicts with ``data`` (numpy,
    [z][y][x] or [y][x]), and optionally ``scale``/``units`` (x calibration),
    ``voltage`` (V) and ``cs`` (mm)."""
    bo = "<" if little_endian else ">"
    image_list = []
    for im in images:
        a = np.asarray(im["data"])
        dims = [("", int(v)) for v in a.shape[::-1]]
        cal = []
        if "scale" in im:
            cal = [("Dimension", [("", [("Origin", 0.0), ("Scale", float(im["scale"])),
                                        ("Units", im.get("units", "nm"))])])]
        data = [("Calibrations", cal), ("Data", a.reshape(-1)), ("DataType", IMAGE_TYPES[a.dtype]),
                ("Dimensions", dims), ("PixelDepth", int(a.dtype.itemsize))]
        tags = []
        if "voltage" in im or "cs" in im:
            mic = []
            if "voltage" in im:
                mic.append(("Voltage", float(im["voltage"])))
            if "cs" in im:
                mic.append(("Cs(mm)", float(im["cs"])))
            tags = [("Microscope Info", mic)]
        image_list.append(("", [("ImageData", data), ("ImageTags", tags), ("Name", "frames")]))
    root = _dir_body([("ApplicationBounds", np.array([0, 0, 100, 100], np.int64)), ("ImageList", image_list)], bo)
    return struct.pack(">IQI", 4, len(root), 1 if little_endian else 0) + root + b"\0" * 8


def write(path, images, little_endian=True):
    with open(path, "wb") as fh:
        fh.write(dm4_bytes(images, little_endian))

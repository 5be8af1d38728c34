"""DM4 movies (zorro_gb300.dm4, the DM4 branch of loadData,
zorro.py:3384-3411): a file assembled byte by byte from the published tag
layout, round trips through an independent writer (oracle/dm4_oracle.py)
in both byte orders and every pixel type the detectors write, and loadData
on a .dm4 movie."""
import struct

import numpy as np
import pytest

from oracle import dm4_oracle
from zorro_gb300 import dm4


def _tag_data(name, info, payload):
    body = b"%%%%" + struct.pack(">Q", len(info)) + b"".join(struct.pack(">Q", v) for v in info) + payload
    return struct.pack(">BH", 21, len(name)) + name + struct.pack(">Q", len(body)) + body


def _tag_dir(name, tags):
    body = struct.pack(">BBQ", 0, 1, len(tags)) + b"".join(tags)
    return struct.pack(">BH", 20, len(name)) + name + struct.pack(">Q", len(body)) + body


def test_known_answer_file():
    """A little-endian DM4 file of one 3 x 2 uint8 image (pixels 1..6, x
    fastest), calibrated at 0.25 nm, with a 200 kV voltage tag."""
    data = _tag_data(b"Data", [20, 10, 6], bytes([1, 2, 3, 4, 5, 6]))
    dtype = _tag_data(b"DataType", [3], struct.pack("<i", 6))
    dims = _tag_dir(b"Dimensions", [_tag_data(b"", [3], struct.pack("<i", 3)),
                                    _tag_data(b"", [3], struct.pack("<i", 2))])
    cal = _tag_dir(b"Calibrations", [_tag_dir(b"Dimension", [_tag_dir(b"", [
        _tag_data(b"Scale", [6], struct.pack("<f", 0.25)),
        _tag_data(b"Units", [20, 4, 2], struct.pack("<2H", ord("n"), ord("m")))])])])
    mic = _tag_dir(b"ImageTags", [_tag_dir(b"Microscope Info", [_tag_data(b"Voltage", [7], struct.pack("<d", 2e5))])])
    image = _tag_dir(b"", [_tag_dir(b"ImageData", [cal, data, dtype, dims]), mic])
    root = struct.pack(">BBQ", 0, 1, 1) + _tag_dir(b"ImageList", [image])
    buf = struct.pack(">IQI", 4, len(root), 1) + root
    ims = dm4.images(dm4.parse(buf))
    assert len(ims) == 1
    assert ims[0]["data"].dtype == np.uint8
    assert np.array_equal(ims[0]["data"], [[1, 2, 3], [4, 5, 6]])
    assert ims[0]["scale"] == pytest.approx(0.25)
    assert ims[0]["units"] == "nm"
    assert ims[0]["voltage"] == 2e5


def test_not_a_dm4_file():
    with pytest.raises(dm4.DM4Error):
        dm4.parse(struct.pack(">IQI", 3, 0, 1) + b"\0" * 16)


@pytest.mark.parametrize("little", [True, False])
@pytest.mark.parametrize("dtype", ["u1", "u2", "i2", "f4"])
def test_round_trip_through_an_independent_writer(tmp_path, little, dtype):
    rng = np.random.default_rng(3)
    movie = (rng.poisson(2.0, (4, 6, 5)) * (1 if dtype != "f4" else 1.5)).astype(dtype)
    thumb = np.zeros((8, 8), dtype="f4")
    path = tmp_path / "movie.dm4"
    dm4_oracle.write(path, [{"data": thumb}, {"data": movie, "scale": 0.105, "units": "nm", "voltage": 300e3,
                                               "cs": 2.7}], little_endian=little)
    frames, info = dm4.read(str(path))
    assert frames.dtype == np.dtype(dtype)
    assert np.array_equal(frames, movie)
    assert info["pixelsize"] == pytest.approx(0.105)
    assert info["voltage"] == pytest.approx(300.0)
    assert info["C3"] == pytest.approx(2.7)


def test_single_image_and_no_units(tmp_path):
    img = np.arange(12, dtype="u2").reshape(3, 4)
    path = tmp_path / "one.dm4"
    dm4_oracle.write(path, [{"data": img, "scale": 1.0, "units": ""}])
    frames, info = dm4.read(str(path))
    assert np.array_equal(frames, img)
    assert info["pixelsize"] is None  # no units: the registrator keeps its pixel size


def test_load_data_reads_a_dm4_movie(tmp_path):
    from zorro_gb300.registrator import ImageRegistrator
    rng = np.random.default_rng(5)
    movie = rng.poisson(1.0, (5, 16, 12)).astype(np.uint8)
    path = tmp_path / "m.dm4"
    dm4_oracle.write(path, [{"data": np.zeros((4, 4), "f4")},
                            {"data": movie, "scale": 0.05, "units": "nm", "voltage": 200e3}])
    reg = ImageRegistrator()
    reg.loadData(str(path))
    assert reg.images.dtype == np.uint8
    assert np.array_equal(reg.images, movie)
    assert reg.pixelsize == pytest.approx(0.05)
    assert reg.voltage == pytest.approx(200.0)

"""Output stage: Camera::radiance_to_rgb tone map (ppm_tone_map) and the
averager2 OpenEXR file (ppm_write_exr), read back field by field."""
import ctypes as C
import math
import struct

import numpy as np

from ppmpa_gb300 import _lib


def test_tone_map_matches_radiance_to_rgb(built_lib):
    lib = _lib.load(built_lib)
    v = np.array([0.0, 1e-9, 0.001, 0.005, 0.00999, 0.01, 0.02, 1.0, 3e-4], np.float64)
    out = np.zeros(len(v), np.int32)
    assert lib.ppm_tone_map(v.ctypes.data_as(C.POINTER(C.c_double)), len(v), 0.01,
                            out.ctypes.data_as(C.POINTER(C.c_int32))) == 0
    want = [math.floor(min(1.0, x / 0.01) ** (1.0 / 2.2) * 255.0) for x in v]
    assert out.tolist() == want
    assert out[5] == 255 and out[0] == 0


def _read_exr(path):
    b = open(path, "rb").read()
    assert struct.unpack_from("<II", b, 0) == (20000630, 2)
    p, attrs = 8, {}
    while b[p] != 0:
        name = b[p:b.index(b"\0", p)].decode(); p += len(name) + 1
        typ = b[p:b.index(b"\0", p)].decode(); p += len(typ) + 1
        (size,) = struct.unpack_from("<I", b, p); p += 4
        attrs[name] = (typ, b[p:p + size]); p += size
    p += 1
    x0, y0, x1, y1 = struct.unpack("<4i", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    offs = struct.unpack_from(f"<{h}Q", b, p)
    img = np.zeros((h, w, 3), np.float32)
    for y, o in enumerate(offs):
        yy, n = struct.unpack_from("<iI", b, o)
        assert yy == y and n == 12 * w
        row = np.frombuffer(b, np.float32, 3 * w, o + 8).reshape(3, w)   # B, G, R
        img[y] = row[::-1].T
    return attrs, img


def test_exr_file_reads_back(built_lib, tmp_path):
    lib = _lib.load(built_lib)
    rng = np.random.default_rng(1)
    img = rng.random((5, 7, 3)) * 0.02
    path = str(tmp_path / "a.exr")
    assert lib.ppm_write_exr(path.encode(), img.ctypes.data_as(C.POINTER(C.c_double)), 7, 5, 100.0) == 0
    attrs, got = _read_exr(path)
    assert list(attrs) == ["channels", "compression", "dataWindow", "displayWindow", "lineOrder",
                           "pixelAspectRatio", "screenWindowCenter", "screenWindowWidth"]
    assert attrs["compression"] == ("compression", b"\0") and attrs["lineOrder"] == ("lineOrder", b"\0")
    assert attrs["channels"][1].startswith(b"B\0\x02\0\0\0")
    assert np.array_equal(got, (img * 100.0).astype(np.float32))

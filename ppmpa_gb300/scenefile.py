"""Scene (*.scene) and camera (*.scr) files through the library's readers
(ppm_scene_parse / ppm_camera_parse of include/ppm_api.h).

load_scene returns an object with the same c_objects / c_materials /
c_lights interface as scene.Scene, so Context.upload_scene and the oracle
take it directly; load_camera starts from the reference camera and applies
the file's settings."""
import ctypes as C
import os

from . import _lib, scene as S


class ParsedScene:
    def __init__(self, objs, mats, lights):
        self._o, self._m, self._l = objs, mats, lights

    @property
    def n_objects(self) -> int:
        return len(self._o)

    @property
    def materials(self):
        return list(self._m)

    @property
    def lights(self):
        return list(self._l)

    def c_objects(self):
        return self._o, len(self._o)

    def c_materials(self):
        return self._m, len(self._m)

    def c_lights(self):
        return self._l, len(self._l)


def _text(path_or_text: str) -> bytes:
    if "\n" not in path_or_text and os.path.exists(path_or_text):
        with open(path_or_text, "rb") as f:
            return f.read()
    return path_or_text.encode()


def load_scene(path_or_text: str) -> ParsedScene:
    lib = _lib.load()
    text = _text(path_or_text)
    no, nm, nl = C.c_int32(0), C.c_int32(0), C.c_int32(0)
    st = lib.ppm_scene_parse(text, None, C.byref(no), None, C.byref(nm), None, C.byref(nl))
    if st != 0:
        raise _lib.PPMError(st, lib.ppm_parse_error().decode())
    objs, mats, lts = (S.Object * no.value)(), (S.Material * nm.value)(), (S.Light * nl.value)()
    st = lib.ppm_scene_parse(text, objs, C.byref(no), mats, C.byref(nm), lts, C.byref(nl))
    if st != 0:
        raise _lib.PPMError(st, lib.ppm_parse_error().decode())
    return ParsedScene(objs, mats, lts)


def load_camera(path_or_text: str, base: S.Camera = None):
    """(Camera, nphoton or None)."""
    lib = _lib.load()
    cam = S.Camera.from_buffer_copy(base if base is not None else S.reference_camera())
    n = C.c_int64(-1)
    st = lib.ppm_camera_parse(_text(path_or_text), C.byref(cam), C.byref(n))
    if st != 0:
        raise _lib.PPMError(st, lib.ppm_parse_error().decode())
    return cam, (n.value if n.value >= 0 else None)

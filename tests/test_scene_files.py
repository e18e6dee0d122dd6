"""Scene and camera file readers (ppm_scene_parse / ppm_camera_parse): the
committed fixtures, written in the reference's file syntax, read back to the
same structs the Python builders make, bit for bit; every example file of
the reference parses (when the reference checkout is at hand); errors carry
the line."""
import ctypes as C
import glob
import os

import pytest

from ppmpa_gb300 import scene as S, scenefile as F
from ppmpa_gb300._lib import PPMError

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout's example/ folder, when one is at hand (the test
# that reads it skips without it)
REF_EXAMPLES = os.environ.get("PPM_REFERENCE_EXAMPLES", "")


def _rows(arr, n):
    return [bytes(C.string_at(C.addressof(arr[i]), C.sizeof(arr[i]))) for i in range(n)]


def test_box_scene_file_equals_builder(built_lib):
    got = F.load_scene(os.path.join(HERE, "golden", "box_c1.scene"))
    want = S.box_scene("c1")
    for part in ("c_objects", "c_materials", "c_lights"):
        a, na = getattr(got, part)()
        b, nb = getattr(want, part)()
        assert na == nb
        assert _rows(a, na) == _rows(b, nb), part


def test_box_camera_file_equals_builder(built_lib):
    cam, nphoton = F.load_camera(os.path.join(HERE, "golden", "box_256.scr"))
    want = S.box_camera(256)
    assert nphoton == 200000
    assert bytes(cam) == bytes(want)


def test_errors_name_the_line(built_lib):
    text = open(os.path.join(HERE, "golden", "box_c1.scene")).read().replace("material: mirror", "material: gold")
    with pytest.raises(PPMError) as e:
        F.load_scene(text)
    assert "unknown material 'gold'" in str(e.value) and "line " in str(e.value)
    with pytest.raises(PPMError):
        F.load_camera("xresolution : 12x\n")


@pytest.mark.skipif(not os.path.isdir(REF_EXAMPLES), reason="reference examples not present")
def test_reference_examples_parse(built_lib):
    import re
    scenes = sorted(glob.glob(os.path.join(REF_EXAMPLES, "*.scene")))
    assert len(scenes) > 10
    parsed = 0
    for path in scenes:
        text = open(path).read()
        # drafts with fields left empty ("reflectance  :") are refused, with the line
        draft = re.search(r"^[ \t]+-?[ \t]*[a-z_]+[ \t]*:[ \t]*$", re.sub(r"#.*", "", text), re.M)
        if draft:
            with pytest.raises(PPMError, match="line "):
                F.load_scene(path)
            continue
        sc = F.load_scene(path)
        parsed += sc.n_objects > 0 and len(sc.lights) > 0     # materials.scene is a material library
    assert parsed > 10
    for path in sorted(glob.glob(os.path.join(REF_EXAMPLES, "*.scr"))):
        cam, n = F.load_camera(path)
        assert cam.xreso > 0 and n and n > 0, path

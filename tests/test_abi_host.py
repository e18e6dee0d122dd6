"""CPU checks of the C ABI library and the host-side logic (no GPU needed):
the library loads and exports every entry point include/ppm_api.h declares;
the host derivations (camera, material) agree bit for bit between the
Python builders, the library and the oracle; error paths return statuses."""
import ctypes as C
import os
import re

import pytest

from oracle import binding as B
from ppmpa_gb300 import _lib, scene as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "ppm_api.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(ppm_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(built_lib)
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding types every declared entry point
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_struct_layouts_match_oracle_and_abi():
    L = B.lib()
    assert C.sizeof(S.Object) == L.orc_sizeof(0) == 120
    assert C.sizeof(S.Material) == L.orc_sizeof(1) == 168
    assert C.sizeof(S.Light) == L.orc_sizeof(2) == 160
    assert C.sizeof(S.Camera) == L.orc_sizeof(3) == 336


def _camera_fields(c):
    return [tuple(getattr(c, f)) for f in ("eye_dir", "origin", "esx", "esy", "eex", "eey")] + [c.photon_power]


@pytest.mark.parametrize("mk", [S.reference_camera, lambda: S.box_camera(512), lambda: S.make_camera(
    320, 200, blur=True, eye_position=(0.3, 1.7, -3.1), target_position=(0.1, 0.9, 2.0), focus=5.5, f_number=2.8)])
def test_camera_derivation_agrees(built_lib, mk):
    lib = _lib.load(built_lib)
    py = mk()
    via_lib = S.Camera.from_buffer_copy(py)
    lib.ppm_camera_derive(C.byref(via_lib))
    via_orc = S.Camera.from_buffer_copy(py)
    B.lib().orc_camera_derive(C.byref(via_orc))
    assert _camera_fields(py) == _camera_fields(via_lib) == _camera_fields(via_orc)


def test_material_derivation_agrees(built_lib):
    lib = _lib.load(built_lib)
    sc = S.reference_scene()
    mats, n = sc.c_materials()
    for i in range(n):
        a = S.Material.from_buffer_copy(mats[i])
        b = S.Material.from_buffer_copy(mats[i])
        lib.ppm_material_derive(C.byref(a))
        B.lib().orc_material_derive(C.byref(b))
        assert a.density_pow == b.density_pow == mats[i].density_pow
        assert a.alpha == b.alpha == mats[i].alpha
    # Surface::new_simple with roughness 0: 1 / (10^5 + 1)
    assert S.new_simple((1, 1, 1), (0, 0, 0), 1, 0, 0).density_pow == 1.0 / (10.0 ** 5.0 + 1.0)


def test_reference_scene_shape():
    sc = S.reference_scene()
    assert len(sc.objects) == 17 and len(sc.materials) == 14 and len(sc.lights) == 1
    assert sc.lights[0].color == (1.0 / 3.0,) * 3
    box = S.box_scene("c2")
    assert len(box.objects) == 7 and box.materials[-1].surface == S.SURF_TS


def test_status_strings_and_no_device_path(built_lib):
    lib = _lib.load(built_lib)
    assert lib.ppm_version() == 1
    assert lib.ppm_status_string(0) == b"ok"
    assert lib.ppm_status_string(3) == b"capacity exceeded"
    assert lib.ppm_ctx_destroy(None) == 0
    # invalid arguments are rejected before any device work
    assert lib.ppm_ctx_create(None, 0, 1) == 1
    assert lib.ppm_scene_upload(None, None, 0, None, 0, None, 0) == 1
    assert lib.ppm_render_step(None, 1) == 1


def test_ctx_create_without_gpu_reports_no_device(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _lib.load(built_lib)
    h = C.c_void_p()
    st = lib.ppm_ctx_create(C.byref(h), 0, 1)
    assert st == 7 and not h.value
    assert lib.ppm_last_error(None).startswith(b"no CUDA device")


def test_cli_usage_and_rust_number_format(built_lib):
    import subprocess
    from ppmpa_gb300 import build as lib_build
    cli = lib_build.CLI
    out = subprocess.run([cli, "-h"], capture_output=True, text=True)
    assert out.returncode == 0 and out.stderr.startswith("Usage: ppmpa [-nc|-h]")
    out = subprocess.run([cli, "1000", "0.1"], capture_output=True, text=True)   # too few arguments
    assert out.returncode == 0 and "Usage" in out.stderr
    # format!("{:e}") and format!("{}") of f64 (shortest round-trip digits)
    vals = ["0.001234", "1.0", "0.0", "123456.0", "0.30000000000000004", "0.01", "250", "4.0", "1e21", "1.5e-7", "-2.5"]
    want = [("1.234e-3", "0.001234"), ("1e0", "1"), ("0e0", "0"), ("1.23456e5", "123456"),
            ("3.0000000000000004e-1", "0.30000000000000004"), ("1e-2", "0.01"), ("2.5e2", "250"), ("4e0", "4"),
            ("1e21", "1000000000000000000000"), ("1.5e-7", "0.00000015"), ("-2.5e0", "-2.5")]
    out = subprocess.run([cli, "--format-test", *vals], capture_output=True, text=True, check=True)
    got = [tuple(l.split()) for l in out.stdout.strip().split("\n")]
    assert got == want


def test_batch_job_layout_matches_header(built_lib):
    """ppm_job: pointer, 2 x int32, 3 pointers with an int32 pair, the render
    config at 48 and the image pointer at 112 (120 bytes)."""
    assert C.sizeof(S.Job) == 120 and S.Job.cfg.offset == 48 and S.Job.image_out.offset == 112
    assert C.sizeof(S.RenderCfg) == 64
    assert C.sizeof(S.Stats) == 360 and S.Stats.photon_rays.offset == 344


def test_every_context_entry_point_rejects_a_null_context(built_lib):
    """Each entry point whose first argument is the context returns
    PPM_ERR_INVALID_ARG for a null context before touching any other
    argument or a device (null pointers and zeros everywhere else)."""
    from ppmpa_gb300 import _lib
    lib = _lib.load()
    skip = {"ppm_ctx_destroy",      # null is a no-op (PPM_OK)
            "ppm_last_error",       # null reads the process-wide message
            "ppm_ctx_stream"}       # returns a pointer, not a status
    checked = 0
    for name, (res, args) in _lib.SIGNATURES.items():
        if name in skip or res is not C.c_int or not args or args[0] is not C.c_void_p:
            continue
        if not name.startswith("ppm_") or name.startswith("ppm_batch"):
            continue
        vals = []
        for t in args[1:]:
            if t in (C.c_double, C.c_float):
                vals.append(0.0)
            elif t in (C.c_int, C.c_int32, C.c_int64, C.c_uint32, C.c_uint64, C.c_size_t):
                vals.append(0)
            else:
                vals.append(None)
        assert getattr(lib, name)(None, *vals) == 1, name
        checked += 1
    assert checked >= 25
    assert lib.ppm_batch_render(None, None, 0, None) == 1


def test_struct_layouts_match_the_header(tmp_path):
    """Every struct of include/ppm_api.h against its ctypes mirror: a C
    program compiled against the header prints each struct's size and each
    field's offset, and the mirrors must agree field by field."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    from ppmpa_gb300 import scene as S
    pairs = {"ppm_object": S.Object, "ppm_material": S.Material, "ppm_light": S.Light, "ppm_camera": S.Camera,
             "ppm_render_cfg": S.RenderCfg, "ppm_stats": S.Stats, "ppm_job": S.Job,
             "ppm_gather_export": S.GatherExport}
    # ctypes field names that differ from the C ones (C keywords / reserved words in Python)
    rename = {("ppm_gather_export", "pass_"): "pass"}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "ppm_api.h"', "int main(void) {"]
    for cname, py in pairs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in py._fields_:
            field = rename.get((cname, f[0]), f[0])
            lines.append(f'printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {field}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([gcc, "-std=c11", "-I", inc, str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n"):
        if line:
            a, b, c = line.split()
            got[(a, b)] = int(c)
    for cname, py in pairs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f in py._fields_:
            assert got[(cname, f[0])] == getattr(py, f[0]).offset, (cname, f[0])

"""ctypes binding of libppmpa_gb300.so (the C ABI of include/ppm_api.h).

The library is required: there is no CPU fallback.  Loading fails loudly if
the CUDA library has not been built (ppmpa_gb300.build.build()).
"""
from __future__ import annotations

import ctypes as C
import os

from . import scene as S

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libppmpa_gb300.so")

_P = C.c_void_p
_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_u8p = C.POINTER(C.c_uint8)
_i8p = C.POINTER(C.c_int8)

# name -> (restype, argtypes); every entry point of include/ppm_api.h
SIGNATURES = {
    "ppm_version": (C.c_int, []),
    "ppm_status_string": (C.c_char_p, [C.c_int]),
    "ppm_ctx_create": (C.c_int, [C.POINTER(_P), C.c_int, C.c_uint64]),
    "ppm_ctx_destroy": (C.c_int, [_P]),
    "ppm_last_error": (C.c_char_p, [_P]),
    "ppm_ctx_stream": (_P, [_P]),
    "ppm_ctx_sync": (C.c_int, [_P]),
    "ppm_scene_upload": (C.c_int, [_P, C.POINTER(S.Object), C.c_int32, C.POINTER(S.Material), C.c_int32,
                                   C.POINTER(S.Light), C.c_int32]),
    "ppm_camera_set": (C.c_int, [_P, C.POINTER(S.Camera)]),
    "ppm_camera_derive": (None, [C.POINTER(S.Camera)]),
    "ppm_material_derive": (None, [C.POINTER(S.Material)]),
    "ppm_intersect": (C.c_int, [_P, _dp, C.c_int64, _dp, _i32p, _dp]),
    "ppm_intersect_f32": (C.c_int, [_P, _dp, C.c_int64, _dp, _i32p]),
    "ppm_trace_photons": (C.c_int, [_P, C.c_int64, C.c_int32, C.c_uint32, _i64p, _dp, _i64p]),
    "ppm_photons_download": (C.c_int, [_P, _dp, _dp, _u8p, _i32p, _i8p, C.c_int64]),
    "ppm_photonmap_build": (C.c_int, [_P, _dp, _dp, _u8p, C.c_int64, C.c_double, C.c_double]),
    "ppm_photonmap_from_trace": (C.c_int, [_P, C.c_double]),
    "ppm_query_within": (C.c_int, [_P, _dp, C.c_int64, _dp, _i64p, _i32p, C.c_int64, _i64p]),
    "ppm_estimate": (C.c_int, [_P, _dp, _dp, C.c_int64, C.c_int32, _dp]),
    "ppm_estimate_noalloc": (C.c_int, [_P, _dp, _dp, C.c_int64, C.c_int32, _dp]),
    "ppm_photonmap_build_f32": (C.c_int, [_P, _fp, _fp, _u8p, C.c_int64, C.c_double, C.c_double]),
    "ppm_query_within_f32": (C.c_int, [_P, _fp, C.c_int64, _dp, _i64p, _i32p, C.c_int64, _i64p]),
    "ppm_estimate_f32": (C.c_int, [_P, _fp, _fp, C.c_int64, _dp, _dp]),
    "ppm_set_accel": (C.c_int, [_P, C.c_int32]),
    "ppm_set_bvh_leaf": (C.c_int, [_P, C.c_int32]),
    "ppm_tune_bvh_leaf": (C.c_int, [_P, _dp, C.c_int64, C.POINTER(C.c_int32), _dp]),
    "ppm_eye_pass": (C.c_int, [_P, C.c_int32, C.c_uint64, C.c_int32, _dp]),
    "ppm_tone_map": (C.c_int, [_dp, C.c_int64, C.c_double, C.POINTER(C.c_int32)]),
    "ppm_write_exr": (C.c_int, [C.c_char_p, _dp, C.c_int32, C.c_int32, C.c_double]),
    "ppm_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_uint64]),
    "ppm_batch_destroy": (C.c_int, [_P]),
    "ppm_batch_last_error": (C.c_char_p, [_P]),
    "ppm_batch_render": (C.c_int, [_P, _P, C.c_int32, _dp]),
    "ppm_batch_set_mode": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "ppm_batch_info": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "ppm_batch_trial_ms": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "ppm_scene_parse": (C.c_int, [C.c_char_p, C.c_void_p, C.POINTER(C.c_int32), C.c_void_p, C.POINTER(C.c_int32),
                                  C.c_void_p, C.POINTER(C.c_int32)]),
    "ppm_camera_parse": (C.c_int, [C.c_char_p, C.c_void_p, C.POINTER(C.c_int64)]),
    "ppm_parse_error": (C.c_char_p, []),
    "ppm_accel_info": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "ppm_photonmap_regrid_f32": (C.c_int, [_P, C.c_double]),
    "ppm_photonmap_tune_f32": (C.c_int, [_P, _fp, _fp, C.c_int64, _dp, _dp, _dp]),
    "ppm_render": (C.c_int, [_P, C.POINTER(S.RenderCfg), _dp]),
    "ppm_render_begin": (C.c_int, [_P, C.POINTER(S.RenderCfg)]),
    "ppm_render_step": (C.c_int, [_P, C.c_int32]),
    "ppm_render_image": (C.c_int, [_P, _dp]),
    "ppm_render_pass_image": (C.c_int, [_P, _dp]),
    "ppm_render_stats": (C.c_int, [_P, C.POINTER(S.Stats)]),
    "ppm_set_stage_timing": (C.c_int, [_P, C.c_int32]),
    "ppm_stage_name": (C.c_char_p, [C.c_int32]),
    "ppm_render_gather_export": (C.c_int, [_P, C.POINTER(S.GatherExport)]),
}

_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load (once) and type the library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build the CUDA library first "
                           "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class PPMError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"ppm status {status}: {msg}")
        self.status = status

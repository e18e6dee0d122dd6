"""ctypes binding of the CPU FP64 oracle (test infrastructure only).

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
reference legs -- never by the product.  The oracle's structs have the same
layout as the C ABI's; scenes are passed as raw bytes of those structs, and
orc_sizeof() is checked against the byte sizes on every call.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None
_dp = C.POINTER(C.c_double)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_u8p = C.POINTER(C.c_uint8)
_i8p = C.POINTER(C.c_int8)
_u32p = C.POINTER(C.c_uint32)


class _Scene(C.Structure):
    _fields_ = [("objs", C.c_void_p), ("n_objs", C.c_int32), ("mats", C.c_void_p), ("n_mats", C.c_int32),
                ("lights", C.c_void_p), ("n_lights", C.c_int32)]


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            path = _build.build()
        L = C.CDLL(path)
        sig = {
            "orc_sizeof": (C.c_int, [C.c_int]),
            "orc_set_libm": (None, [C.c_int]),
            "orc_set_threads": (None, [C.c_int]),
            "orc_get_threads": (C.c_int, []),
            "orc_normalize": (C.c_int, [_dp, _dp]),
            "orc_filter_cone": (C.c_double, [C.c_double, C.c_double]),
            "orc_filter_gauss": (C.c_double, [C.c_double, C.c_double]),
            "orc_filter_gauss_corr": (C.c_double, [C.c_double, C.c_double, C.c_double]),
            "orc_check_under": (C.c_int, [_dp, C.c_int, C.c_double]),
            "orc_color_normalize": (None, [_dp, _dp]),
            "orc_decide_wavelength": (C.c_int, [_dp, C.c_double]),
            "orc_schlick": (C.c_double, [C.c_double, C.c_double]),
            "orc_relative_ior": (C.c_double, [C.c_double, C.c_double]),
            "orc_ray_target": (None, [_dp, _dp, C.c_double, _dp]),
            "orc_new_dir": (C.c_int, [C.c_double, C.c_double, C.c_double, _dp]),
            "orc_get_normal": (C.c_int, [C.c_void_p, _dp, _dp]),
            "orc_material_derive": (None, [C.c_void_p]),
            "orc_camera_derive": (None, [C.c_void_p]),
            "orc_pm_sin": (C.c_double, [C.c_double]),
            "orc_pm_cos": (C.c_double, [C.c_double]),
            "orc_pm_exp": (C.c_double, [C.c_double]),
            "orc_pm_log": (C.c_double, [C.c_double]),
            "orc_philox": (None, [_u32p, _u32p, _u32p]),
            "orc_intersect": (None, [C.POINTER(_Scene), _dp, C.c_int64, _dp, _i32p, _dp, _i32p]),
            "orc_within": (C.c_int64, [_dp, C.c_int64, _dp, C.c_int64, _dp, _i64p, _i32p, C.c_int64]),
            "orc_estimate": (None, [_dp, _dp, _u8p, C.c_int64, _dp, _dp, C.c_int64, C.c_double, C.c_double,
                                    C.c_int, _dp]),
            "orc_estimate_radii": (None, [_dp, _dp, _u8p, C.c_int64, _dp, _dp, C.c_int64, _dp, C.c_double,
                                          C.c_int, _dp]),
            "orc_last_query_seconds": (C.c_double, []),
            "orc_gather_sums": (None, [_dp, _dp, _u8p, C.c_int64, _dp, _dp, C.c_int64, C.c_double, C.c_int,
                                       _i64p, C.POINTER(C.c_uint64), _dp]),
            "orc_trace_photons": (C.c_int64, [C.POINTER(_Scene), C.c_int64, C.c_int, C.c_uint64, C.c_uint32,
                                              _dp, _dp, _u8p, _i32p, _i8p, C.c_int64, _dp, _i64p]),
            "orc_classic_pass": (None, [C.POINTER(_Scene), C.c_void_p, C.c_uint64, C.c_uint32, _dp]),
            "orc_eye_pass": (None, [C.POINTER(_Scene), C.c_void_p, _dp, _dp, _u8p, C.c_int64, C.c_double,
                                    C.c_double, C.c_int, C.c_uint64, C.c_uint32, _dp]),
            "orc_render": (None, [C.POINTER(_Scene), C.c_void_p, C.c_int64, C.c_int, C.c_double, C.c_double,
                                  C.c_int, C.c_int, C.c_uint64, _dp]),
            "orc_radius_schedule": (None, [C.c_double, C.c_double, C.c_int, C.c_int, _dp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype, fn.argtypes = res, args
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


class Oracle:
    """Numpy-level access to the FP64 restatement for one scene."""

    def __init__(self, scene, camera=None, threads: int = 0, libm: bool = False):
        L = lib()
        self.L = L
        objs, no = scene.c_objects()
        mats, nm = scene.c_materials()
        lts, nl = scene.c_lights()
        for which, (arr, n) in enumerate(((objs, no), (mats, nm), (lts, nl))):
            if n and C.sizeof(arr) // len(arr) != L.orc_sizeof(which):
                raise RuntimeError("oracle struct layout differs from the C ABI")
        self._keep = (objs, mats, lts)
        self.sc = _Scene(C.cast(objs, C.c_void_p), no, C.cast(mats, C.c_void_p), nm, C.cast(lts, C.c_void_p), nl)
        self.camera = camera
        if camera is not None and C.sizeof(camera) != L.orc_sizeof(3):
            raise RuntimeError("oracle camera layout differs from the C ABI")
        L.orc_set_threads(int(threads))
        L.orc_set_libm(int(bool(libm)))

    def intersect(self, rays):
        rays = np.ascontiguousarray(rays, np.float64).reshape(-1, 6)
        n = rays.shape[0]
        t = np.zeros(n)
        obj = np.zeros(n, np.int32)
        nrm = np.zeros((n, 3))
        io = np.zeros(n, np.int32)
        self.L.orc_intersect(C.byref(self.sc), _p(rays, C.c_double), n, _p(t, C.c_double), _p(obj, C.c_int32),
                             _p(nrm, C.c_double), _p(io, C.c_int32))
        return t, obj, nrm, io

    def trace_photons(self, nphoton: int, use_classic: bool = True, seed: int = 1, pass_index: int = 0) -> dict:
        cap = int(nphoton) * 10 + 64
        pos = np.zeros((cap, 3))
        dirs = np.zeros((cap, 3))
        wl = np.zeros(cap, np.uint8)
        emit = np.zeros(cap, np.int32)
        level = np.zeros(cap, np.int8)
        pw = C.c_double()
        nem = C.c_int64()
        n = self.L.orc_trace_photons(C.byref(self.sc), int(nphoton), int(bool(use_classic)), int(seed),
                                     int(pass_index), _p(pos, C.c_double), _p(dirs, C.c_double), _p(wl, C.c_uint8),
                                     _p(emit, C.c_int32), _p(level, C.c_int8), cap, C.byref(pw), C.byref(nem))
        if n < 0:
            raise RuntimeError("oracle photon buffer too small")
        return dict(pos=pos[:n], dir=dirs[:n], wl=wl[:n], emit=emit[:n], level=level[:n], power=pw.value,
                    n_emitted=nem.value)

    def within(self, ppos, q, r2, cap_hint: int = 0):
        """In-radius sets (offsets, ascending indices).  With cap_hint >= the
        total, one call (one grid build) counts and fills."""
        ppos = np.ascontiguousarray(ppos, np.float64).reshape(-1, 3)
        q = np.ascontiguousarray(q, np.float64).reshape(-1, 3)
        r2 = np.ascontiguousarray(np.broadcast_to(np.asarray(r2, np.float64), (q.shape[0],)))
        off = np.zeros(q.shape[0] + 1, np.int64)
        idx = np.zeros(max(1, cap_hint), np.int32)
        tot = self.L.orc_within(_p(ppos, C.c_double), ppos.shape[0], _p(q, C.c_double), q.shape[0],
                                _p(r2, C.c_double), _p(off, C.c_int64), _p(idx, C.c_int32) if cap_hint else None,
                                cap_hint)
        if tot > cap_hint:
            idx = np.zeros(max(1, tot), np.int32)
            self.L.orc_within(_p(ppos, C.c_double), ppos.shape[0], _p(q, C.c_double), q.shape[0],
                              _p(r2, C.c_double), _p(off, C.c_int64), _p(idx, C.c_int32), idx.size)
        return off, idx[:tot]

    def estimate_radii(self, ppos, pdir, pwl, qpos, qnrm, r2, pw, pfilter=0):
        """estimate with one radius^2 per query."""
        ppos = np.ascontiguousarray(ppos, np.float64).reshape(-1, 3)
        pdir = np.ascontiguousarray(pdir, np.float64).reshape(-1, 3)
        pwl = np.ascontiguousarray(pwl, np.uint8)
        qpos = np.ascontiguousarray(qpos, np.float64).reshape(-1, 3)
        qnrm = np.ascontiguousarray(qnrm, np.float64).reshape(-1, 3)
        r2 = np.ascontiguousarray(np.broadcast_to(np.asarray(r2, np.float64), (qpos.shape[0],)))
        rgb = np.zeros((qpos.shape[0], 3))
        self.L.orc_estimate_radii(_p(ppos, C.c_double), _p(pdir, C.c_double), _p(pwl, C.c_uint8), ppos.shape[0],
                                  _p(qpos, C.c_double), _p(qnrm, C.c_double), qpos.shape[0], _p(r2, C.c_double),
                                  float(pw), int(pfilter), _p(rgb, C.c_double))
        return rgb

    def gather_sums(self, ppos, pdir, pwl, qpos, qnrm, r2, pfilter=0):
        """Per query: photons within r2, their set checksum and the flux sums of
        estimate_radiance before pw and 1/(pi r2) (orc_gather_sums)."""
        ppos = np.ascontiguousarray(ppos, np.float64).reshape(-1, 3)
        pdir = np.ascontiguousarray(pdir, np.float64).reshape(-1, 3)
        pwl = np.ascontiguousarray(pwl, np.uint8)
        qpos = np.ascontiguousarray(qpos, np.float64).reshape(-1, 3)
        qnrm = np.ascontiguousarray(qnrm, np.float64).reshape(-1, 3)
        nq = qpos.shape[0]
        count = np.zeros(nq, np.int64)
        check = np.zeros(nq, np.uint64)
        sums = np.zeros((nq, 3))
        self.L.orc_gather_sums(_p(ppos, C.c_double), _p(pdir, C.c_double), _p(pwl, C.c_uint8), ppos.shape[0],
                               _p(qpos, C.c_double), _p(qnrm, C.c_double), nq, float(r2), int(pfilter),
                               _p(count, C.c_int64), _p(check, C.c_uint64), _p(sums, C.c_double))
        return count, check, sums

    def estimate(self, ppos, pdir, pwl, qpos, qnrm, r2, pw, pfilter=0):
        ppos = np.ascontiguousarray(ppos, np.float64).reshape(-1, 3)
        pdir = np.ascontiguousarray(pdir, np.float64).reshape(-1, 3)
        pwl = np.ascontiguousarray(pwl, np.uint8)
        qpos = np.ascontiguousarray(qpos, np.float64).reshape(-1, 3)
        qnrm = np.ascontiguousarray(qnrm, np.float64).reshape(-1, 3)
        rgb = np.zeros((qpos.shape[0], 3))
        self.L.orc_estimate(_p(ppos, C.c_double), _p(pdir, C.c_double), _p(pwl, C.c_uint8), ppos.shape[0],
                            _p(qpos, C.c_double), _p(qnrm, C.c_double), qpos.shape[0], float(r2), float(pw),
                            int(pfilter), _p(rgb, C.c_double))
        return rgb

    def eye_pass(self, photons: dict, r2: float, use_classic: bool = True, seed: int = 1, pass_index: int = 0):
        cam = self.camera
        img = np.zeros((cam.yreso, cam.xreso, 3))
        pos = np.ascontiguousarray(photons["pos"], np.float64)
        dirs = np.ascontiguousarray(photons["dir"], np.float64)
        wl = np.ascontiguousarray(photons["wl"], np.uint8)
        self.L.orc_eye_pass(C.byref(self.sc), C.byref(cam), _p(pos, C.c_double), _p(dirs, C.c_double),
                            _p(wl, C.c_uint8), pos.shape[0], float(r2), float(photons["power"]),
                            int(bool(use_classic)), int(seed), int(pass_index), _p(img, C.c_double))
        return img

    def classic_pass(self, seed: int = 1, pass_index: int = 0):
        """One pass of trace_ray_classic over the camera's pixels."""
        cam = self.camera
        img = np.zeros((cam.yreso, cam.xreso, 3))
        self.L.orc_classic_pass(C.byref(self.sc), C.byref(cam), int(seed), int(pass_index), _p(img, C.c_double))
        return img

    def render(self, nphoton, passes, r0, alpha, schedule_offset=1, use_classic=True, seed=1):
        cam = self.camera
        img = np.zeros((cam.yreso, cam.xreso, 3))
        self.L.orc_render(C.byref(self.sc), C.byref(cam), int(nphoton), int(passes), float(r0), float(alpha),
                          int(schedule_offset), int(bool(use_classic)), int(seed), _p(img, C.c_double))
        return img


def radius_schedule(r0, alpha, offset, passes):
    out = np.zeros(passes)
    lib().orc_radius_schedule(float(r0), float(alpha), int(offset), int(passes), _p(out, C.c_double))
    return out

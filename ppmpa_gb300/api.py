"""Python host interface over the C ABI, mirroring the reference's operators.

    Context.trace_photons     <- trace_photon over all lights   (src/tracer.rs:31, src/bin/ppmpa.rs:86-92)
    Context.build_photonmap   <- build_photonmap                (src/photonmap.rs:23-29)
    Context.query_within      <- kdtree.within(p, r2, squared_euclidean) (src/tracer.rs:180)
    Context.estimate          <- estimate_radiance              (src/tracer.rs:179-195)
    Context.intersect         <- calc_intersection              (src/tracer.rs:306-350)
    Context.render            <- ppmpa passes + PA schedule + averaging
                                 (src/bin/ppmpa.rs:74-84, util/iterator.rb:33-38, util/averager.rb:66-69)

Errors come back as PPMError (the ABI never throws).  Every compute call runs
on the GPU through libppmpa_gb300.so.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import scene as S
from ._lib import PPMError, load

PLAIN, MIXED = 0, 1


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype)) if a is not None else None


# RenderConfig.flags bits (include/ppm_api.h)
RENDER_TUNE_CELLS = 1   # time 1 to 4 cells per radius before the render, keep the fastest
RENDER_CLASSIC = 2      # the classic ray tracer (trace_ray_classic) instead of photon mapping
RENDER_TILE_GATHER = 4  # mixed render: the tile gather (32 hit points per warp) instead of the row walk

# Batch.set_mode modes (include/ppm_api.h)
BATCH_AUTO, BATCH_STAGED, BATCH_GRAPHS = 0, 1, 2


@dataclass
class RenderConfig:
    nphoton: int = 200_000
    passes: int = 10
    use_classic: bool = True
    radius0: float = 0.05
    alpha: float = 0.7
    schedule_offset: int = 1
    precision: int = MIXED
    use_graph: bool = True
    cell_factor: int = 0
    seed: int = 1
    first_pass: int = 0
    flags: int = 0

    def to_c(self) -> S.RenderCfg:
        c = S.RenderCfg()
        c.nphoton, c.passes, c.use_classic = int(self.nphoton), int(self.passes), int(bool(self.use_classic))
        c.radius0, c.alpha, c.schedule_offset = float(self.radius0), float(self.alpha), int(self.schedule_offset)
        c.precision, c.use_graph, c.cell_factor = int(self.precision), int(bool(self.use_graph)), int(self.cell_factor)
        c.seed, c.first_pass, c.flags = int(self.seed), int(self.first_pass), int(self.flags)
        return c


class Context:
    """One GPU context (ppm_ctx): scene, camera, photon map and render state."""

    def __init__(self, device: int = 0, seed: int = 1):
        self.lib = load()
        h = C.c_void_p()
        st = self.lib.ppm_ctx_create(C.byref(h), int(device), int(seed))
        if st != 0:
            raise PPMError(st, self.lib.ppm_last_error(None).decode())
        self.h = h
        self.camera = None
        self.seed = seed

    # -- plumbing ------------------------------------------------------------
    def _check(self, st: int):
        if st != 0:
            raise PPMError(st, self.lib.ppm_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.ppm_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def stream(self) -> int:
        return int(self.lib.ppm_ctx_stream(self.h) or 0)

    def sync(self):
        self._check(self.lib.ppm_ctx_sync(self.h))

    # -- input -----------------------------------------------------------------
    def upload_scene(self, sc: S.Scene):
        objs, no = sc.c_objects()
        mats, nm = sc.c_materials()
        lts, nl = sc.c_lights()
        self._check(self.lib.ppm_scene_upload(self.h, objs, no, mats, nm, lts, nl))

    def set_camera(self, cam: S.Camera):
        self._check(self.lib.ppm_camera_set(self.h, C.byref(cam)))
        self.camera = cam

    # -- parity operators ----------------------------------------------------------
    def intersect(self, rays: np.ndarray, f32: bool = False):
        rays = np.ascontiguousarray(rays, dtype=np.float64).reshape(-1, 6)
        n = rays.shape[0]
        t = np.zeros(n, np.float64)
        obj = np.zeros(n, np.int32)
        if f32:
            self._check(self.lib.ppm_intersect_f32(self.h, _ptr(rays, C.c_double), n, _ptr(t, C.c_double),
                                                   _ptr(obj, C.c_int32)))
            return t, obj
        nrm = np.zeros((n, 3), np.float64)
        self._check(self.lib.ppm_intersect(self.h, _ptr(rays, C.c_double), n, _ptr(t, C.c_double),
                                           _ptr(obj, C.c_int32), _ptr(nrm, C.c_double)))
        return t, obj, nrm

    def trace_photons(self, nphoton: int, use_classic: bool = True, pass_index: int = 0) -> dict:
        ns, nem, pw = C.c_int64(), C.c_int64(), C.c_double()
        self._check(self.lib.ppm_trace_photons(self.h, int(nphoton), int(bool(use_classic)), int(pass_index),
                                               C.byref(ns), C.byref(pw), C.byref(nem)))
        n = ns.value
        pos = np.zeros((n, 3), np.float64)
        dirs = np.zeros((n, 3), np.float64)
        wl = np.zeros(n, np.uint8)
        emit = np.zeros(n, np.int32)
        level = np.zeros(n, np.int8)
        self._check(self.lib.ppm_photons_download(self.h, _ptr(pos, C.c_double), _ptr(dirs, C.c_double),
                                                  _ptr(wl, C.c_uint8), _ptr(emit, C.c_int32),
                                                  _ptr(level, C.c_int8), n))
        return dict(pos=pos, dir=dirs, wl=wl, emit=emit, level=level, power=pw.value, n_emitted=nem.value)

    def build_photonmap(self, pos, dirs, wl, power: float, radius2: float):
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        dirs = np.ascontiguousarray(dirs, np.float64).reshape(-1, 3)
        wl = np.ascontiguousarray(wl, np.uint8)
        self._check(self.lib.ppm_photonmap_build(self.h, _ptr(pos, C.c_double), _ptr(dirs, C.c_double),
                                                 _ptr(wl, C.c_uint8), pos.shape[0], float(power), float(radius2)))

    def photonmap_from_trace(self, radius2: float):
        self._check(self.lib.ppm_photonmap_from_trace(self.h, float(radius2)))

    def query_within(self, q, r2):
        q = np.ascontiguousarray(q, np.float64).reshape(-1, 3)
        nq = q.shape[0]
        r2 = np.ascontiguousarray(np.broadcast_to(np.asarray(r2, np.float64), (nq,)))
        off = np.zeros(nq + 1, np.int64)
        tot = C.c_int64()
        self._check(self.lib.ppm_query_within(self.h, _ptr(q, C.c_double), nq, _ptr(r2, C.c_double),
                                              _ptr(off, C.c_int64), None, 0, C.byref(tot)))
        idx = np.zeros(max(1, tot.value), np.int32)
        self._check(self.lib.ppm_query_within(self.h, _ptr(q, C.c_double), nq, _ptr(r2, C.c_double),
                                              _ptr(off, C.c_int64), _ptr(idx, C.c_int32), idx.size, C.byref(tot)))
        return off, idx[:tot.value]

    def estimate(self, pos, nrm, pfilter: int = S.FILTER_NONE):
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        nrm = np.ascontiguousarray(nrm, np.float64).reshape(-1, 3)
        rgb = np.zeros((pos.shape[0], 3), np.float64)
        self._check(self.lib.ppm_estimate(self.h, _ptr(pos, C.c_double), _ptr(nrm, C.c_double), pos.shape[0],
                                          int(pfilter), _ptr(rgb, C.c_double)))
        return rgb

    # -- FP32 photon map -------------------------------------------------------------
    def build_photonmap_f32(self, pos, dirs, wl, power: float, radius2_max: float):
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        dirs = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        wl = np.ascontiguousarray(wl, np.uint8)
        self._check(self.lib.ppm_photonmap_build_f32(self.h, _ptr(pos, C.c_float), _ptr(dirs, C.c_float),
                                                     _ptr(wl, C.c_uint8), pos.shape[0], float(power),
                                                     float(radius2_max)))

    def query_within_f32(self, q, r2, count_only: bool = False):
        """(offsets, indices); with count_only the offsets alone (sizes of the sets)."""
        q = np.ascontiguousarray(q, np.float32).reshape(-1, 3)
        nq = q.shape[0]
        r2 = np.ascontiguousarray(np.broadcast_to(np.asarray(r2, np.float64), (nq,)))
        off = np.zeros(nq + 1, np.int64)
        tot = C.c_int64()
        self._check(self.lib.ppm_query_within_f32(self.h, _ptr(q, C.c_float), nq, _ptr(r2, C.c_double),
                                                  _ptr(off, C.c_int64), None, 0, C.byref(tot)))
        if count_only:
            return off, None
        idx = np.zeros(max(1, tot.value), np.int32)
        self._check(self.lib.ppm_query_within_f32(self.h, _ptr(q, C.c_float), nq, _ptr(r2, C.c_double),
                                                  _ptr(off, C.c_int64), _ptr(idx, C.c_int32), idx.size,
                                                  C.byref(tot)))
        return off, idx[:tot.value]

    def estimate_f32(self, pos, nrm, r2):
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        nrm = np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
        nq = pos.shape[0]
        r2 = np.ascontiguousarray(np.broadcast_to(np.asarray(r2, np.float64), (nq,)))
        rgb = np.zeros((nq, 3), np.float64)
        self._check(self.lib.ppm_estimate_f32(self.h, _ptr(pos, C.c_float), _ptr(nrm, C.c_float), nq,
                                              _ptr(r2, C.c_double), _ptr(rgb, C.c_double)))
        return rgb

    def set_accel(self, mode: int):
        """0 automatic (BVH from 32 bounded objects), 1 BVH, 2 loop over the objects."""
        self._check(self.lib.ppm_set_accel(self.h, int(mode)))

    def set_bvh_leaf(self, leaf_max: int):
        self._check(self.lib.ppm_set_bvh_leaf(self.h, int(leaf_max)))

    def tune_bvh_leaf(self, rays):
        """Picks the BVH leaf size (1, 2, 4, 8) fastest for these rays (n x 6); returns (leaf, ms)."""
        rays = np.ascontiguousarray(rays, np.float64).reshape(-1, 6)
        leaf, ms = C.c_int32(), C.c_double()
        self._check(self.lib.ppm_tune_bvh_leaf(self.h, _ptr(rays, C.c_double), rays.shape[0], C.byref(leaf),
                                               C.byref(ms)))
        return leaf.value, ms.value

    def accel_info(self) -> dict:
        m, u = C.c_int32(), C.c_int32()
        self._check(self.lib.ppm_accel_info(self.h, C.byref(m), C.byref(u)))
        return dict(bvh_objects=m.value, unbounded=u.value)

    def regrid_photonmap_f32(self, cells_per_radius: float):
        self._check(self.lib.ppm_photonmap_regrid_f32(self.h, float(cells_per_radius)))

    def tune_photonmap_f32(self, pos, nrm, r2):
        """Picks the FP32 map's cell size for these queries; returns (cells per radius, ms)."""
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        nrm = np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
        nq = pos.shape[0]
        r2 = np.ascontiguousarray(np.broadcast_to(np.asarray(r2, np.float64), (nq,)))
        best, ms = C.c_double(), C.c_double()
        self._check(self.lib.ppm_photonmap_tune_f32(self.h, _ptr(pos, C.c_float), _ptr(nrm, C.c_float), nq,
                                                    _ptr(r2, C.c_double), C.byref(best), C.byref(ms)))
        return best.value, ms.value

    # -- progressive render ------------------------------------------------------------
    def _image_shape(self):
        if self.camera is None:
            raise PPMError(6, "no camera set (set_camera before rendering)")
        return (self.camera.yreso, self.camera.xreso, 3)

    def render(self, cfg: RenderConfig) -> np.ndarray:
        img = np.zeros(self._image_shape(), np.float64)
        c = cfg.to_c()
        self._check(self.lib.ppm_render(self.h, C.byref(c), _ptr(img, C.c_double)))
        return img

    def render_begin(self, cfg: RenderConfig):
        c = cfg.to_c()
        self._check(self.lib.ppm_render_begin(self.h, C.byref(c)))

    def render_step(self, npasses: int = 1):
        self._check(self.lib.ppm_render_step(self.h, int(npasses)))

    def render_image(self) -> np.ndarray:
        img = np.zeros(self._image_shape(), np.float64)
        self._check(self.lib.ppm_render_image(self.h, _ptr(img, C.c_double)))
        return img

    def render_pass_image(self) -> np.ndarray:
        img = np.zeros(self._image_shape(), np.float64)
        self._check(self.lib.ppm_render_pass_image(self.h, _ptr(img, C.c_double)))
        return img

    def render_gather_export(self) -> dict:
        """Runs one more pass of the begun mixed render with the gather's
        per-hit-point records on (ppm_render_gather_export) and returns that
        pass's sorted photon map (float32 n x 4; the last column holds the
        direction word's bits), hit points (float32 n x 10; the pixel's bits in
        the last column), per-hit-point FP32 flux sums, in-radius counts,
        neighbour-set checksums and the FP32 gathered-flux image."""
        ex = S.GatherExport()
        self._check(self.lib.ppm_render_gather_export(self.h, C.byref(ex)))   # capacities only
        ph = np.zeros((ex.n_photons, 4), np.float32)
        hits = np.zeros((ex.n_hits, 10), np.float32)
        sums = np.zeros((ex.n_hits, 3), np.float32)
        counts = np.zeros(ex.n_hits, np.uint32)
        checks = np.zeros(ex.n_hits, np.uint64)
        gathered = np.zeros(self._image_shape(), np.float32)
        ex.photon_cap, ex.hit_cap = ph.shape[0], hits.shape[0]
        ex.photons, ex.hits, ex.sums = _ptr(ph, C.c_float), _ptr(hits, C.c_float), _ptr(sums, C.c_float)
        ex.counts, ex.checksums = _ptr(counts, C.c_uint32), _ptr(checks, C.c_uint64)
        ex.gathered = _ptr(gathered, C.c_float)
        self._check(self.lib.ppm_render_gather_export(self.h, C.byref(ex)))
        n, m = ex.n_photons, ex.n_hits
        return dict(photons=ph[:n].copy(), hits=hits[:m].copy(), sums=sums[:m].copy(), counts=counts[:m].copy(),
                    checksums=checks[:m].copy(), gathered=gathered, radius2=ex.radius2,
                    photon_power=ex.photon_power, pass_index=ex.pass_, pfilter=ex.pfilter)

    def set_stage_timing(self, on):
        """0 off, 1 per-stage CUDA events, 2 events + gather candidate counters."""
        self._check(self.lib.ppm_set_stage_timing(self.h, int(on)))

    def stats(self) -> dict:
        s = S.Stats()
        self._check(self.lib.ppm_render_stats(self.h, C.byref(s)))
        names = [self.lib.ppm_stage_name(i).decode() for i in range(s.n_stages)]
        return dict(photons_emitted=s.photons_emitted, photons_stored=s.photons_stored, hit_points=s.hit_points,
                    grid_cells=s.grid_cells, passes_done=s.passes_done, kernels_per_pass=s.kernels_per_pass,
                    r2=s.r2, candidates=s.candidates, in_radius=s.in_radius, gather_slots=s.gather_slots,
                    cell_factor=s.cell_factor, photon_rays=s.photon_rays, eye_rays=s.eye_rays,
                    stage_ms={n: s.stage_ms[i] for i, n in enumerate(names)},
                    stage_calls={n: s.stage_calls[i] for i, n in enumerate(names)})


class Batch:
    """Many independent renders on one GPU (ppm_batch): one graph launch per
    pass runs a pass of every job."""

    def __init__(self, device: int = 0, seed: int = 1):
        self.lib = load()
        h = C.c_void_p()
        st = self.lib.ppm_batch_create(C.byref(h), int(device), int(seed))
        if st != 0:
            raise PPMError(st, self.lib.ppm_last_error(None).decode())
        self.h = h

    def close(self):
        if self.h:
            self.lib.ppm_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_mode(self, mode: int = 0, tile: int = 0):
        """BATCH_AUTO / BATCH_STAGED (one launch per stage over every job) /
        BATCH_GRAPHS (the jobs' pass graphs side by side); tile: photons per
        map-build work item of the staged passes (0: tuned per render)."""
        st = self.lib.ppm_batch_set_mode(self.h, int(mode), int(tile))
        if st != 0:
            raise PPMError(st, "bad batch mode")

    def info(self) -> dict:
        """How the last render ran (staged or graphs, the tile) and, after
        an AUTO render, the ms per pass its trial measured for each mode."""
        staged, tile = C.c_int32(), C.c_int32()
        self.lib.ppm_batch_info(self.h, C.byref(staged), C.byref(tile))
        out = dict(staged=bool(staged.value), tile=tile.value)
        s_ms, g_ms = C.c_double(), C.c_double()
        if self.lib.ppm_batch_trial_ms(self.h, C.byref(s_ms), C.byref(g_ms)) == 0:
            out["trial_ms"] = dict(staged=s_ms.value, graphs=g_ms.value)
        return out

    def render(self, jobs):
        """jobs: [(scene, camera, RenderConfig)]; returns ([images], device ms of the passes)."""
        arr = (S.Job * max(1, len(jobs)))()
        keep, images = [], []
        for j, (sc, cam, cfg) in enumerate(jobs):
            objs, no = sc.c_objects()
            mats, nm = sc.c_materials()
            lts, nl = sc.c_lights()
            img = np.zeros((cam.yreso, cam.xreso, 3), np.float64)
            cam_c = S.Camera.from_buffer_copy(cam)
            keep += [objs, mats, lts, cam_c]
            images.append(img)
            jb = arr[j]
            jb.objs, jb.n_objs = C.cast(objs, C.c_void_p), no
            jb.mats, jb.n_mats = C.cast(mats, C.c_void_p), nm
            jb.lights, jb.n_lights = C.cast(lts, C.c_void_p), nl
            jb.cam = C.cast(C.pointer(cam_c), C.c_void_p)
            jb.cfg = cfg.to_c()
            jb.image_out = _ptr(img, C.c_double)
        ms = C.c_double()
        st = self.lib.ppm_batch_render(self.h, arr, len(jobs), C.byref(ms))
        if st != 0:
            raise PPMError(st, self.lib.ppm_batch_last_error(self.h).decode())
        return images, ms.value

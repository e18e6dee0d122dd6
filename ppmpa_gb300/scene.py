"""Scene, material, light and camera descriptions (host side of the C ABI).

The ctypes structures mirror include/ppm_api.h field for field.  The builder
functions mirror the reference's constructors so a scene written against the
reference reads the same here:

  Shape::Plain / Sphere / new_polygon / new_parallelogram  (src/ray/geometry.rs:66-115)
  Surface::new_simple / new_ts                              (src/ray/surface.rs:45-66)
  Material {emittance, transmittance, ior, surface}         (src/ray/material.rs:11-16)
  Light::PointLight / ParallelogramLight / SunLight         (src/ray/light.rs:16-39)
  read_scene / read_camera defaults                          (src/scene.rs:20-448, src/camera.rs:108-206)

All vector arithmetic here is plain IEEE double in the reference's
evaluation order, so derived normals equal the reference's bit for bit.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import List, Sequence

D3 = C.c_double * 3

SHAPE_POINT, SHAPE_PLAIN, SHAPE_SPHERE, SHAPE_POLYGON, SHAPE_PARALLELOGRAM = 0, 1, 2, 3, 4
SURF_NOTHING, SURF_SIMPLE, SURF_TS = 0, 1, 2
LIGHT_POINT, LIGHT_PARALLELOGRAM, LIGHT_SUN, LIGHT_SPOT = 0, 1, 2, 3
FILTER_NONE, FILTER_CONE, FILTER_GAUSS = 0, 1, 2
WL_RED, WL_GREEN, WL_BLUE = 0, 1, 2


class Object(C.Structure):
    _fields_ = [("shape", C.c_int32), ("material", C.c_int32), ("position", D3), ("nvec", D3),
                ("dir1", D3), ("dir2", D3), ("dist", C.c_double), ("radius", C.c_double)]


class Material(C.Structure):
    _fields_ = [("emittance", D3), ("transmittance", D3), ("ior", D3), ("surface", C.c_int32),
                ("pad_", C.c_int32), ("color_diff", D3), ("color_spec", D3), ("scatter", C.c_double),
                ("metalness", C.c_double), ("roughness", C.c_double), ("density_pow", C.c_double),
                ("alpha", C.c_double)]


class Light(C.Structure):
    _fields_ = [("kind", C.c_int32), ("pad_", C.c_int32), ("color", D3), ("flux", C.c_double),
                ("pos", D3), ("nvec", D3), ("dir1", D3), ("dir2", D3), ("dir", D3)]


class Camera(C.Structure):
    _fields_ = [("xreso", C.c_int32), ("yreso", C.c_int32), ("progressive", C.c_int32),
                ("antialias", C.c_int32), ("blur", C.c_int32), ("use_classic", C.c_int32),
                ("pfilter", C.c_int32), ("n_sample_photon", C.c_int32),
                ("radius", C.c_double), ("max_radiance", C.c_double), ("iso_sens", C.c_double),
                ("shut_speed", C.c_double), ("focal_len", C.c_double), ("f_number", C.c_double),
                ("focus", C.c_double), ("ambient", D3), ("eye_pos", D3), ("target", D3), ("upper", D3),
                ("eye_dir", D3), ("origin", D3), ("esx", D3), ("esy", D3), ("eex", D3), ("eey", D3),
                ("photon_power", C.c_double)]


class RenderCfg(C.Structure):
    _fields_ = [("nphoton", C.c_int64), ("passes", C.c_int32), ("use_classic", C.c_int32),
                ("radius0", C.c_double), ("alpha", C.c_double), ("schedule_offset", C.c_int32),
                ("precision", C.c_int32), ("use_graph", C.c_int32), ("cell_factor", C.c_int32),
                ("seed", C.c_uint64), ("first_pass", C.c_int32), ("flags", C.c_int32)]


class Job(C.Structure):
    """ppm_job: one render of a batch (scene arrays, camera, config, output image)."""
    _fields_ = [("objs", C.c_void_p), ("n_objs", C.c_int32), ("n_mats", C.c_int32), ("mats", C.c_void_p),
                ("lights", C.c_void_p), ("n_lights", C.c_int32), ("pad_", C.c_int32), ("cam", C.c_void_p),
                ("cfg", RenderCfg), ("image_out", C.POINTER(C.c_double))]


class Stats(C.Structure):
    _fields_ = [("photons_emitted", C.c_int64), ("photons_stored", C.c_int64), ("hit_points", C.c_int64),
                ("grid_cells", C.c_int64), ("passes_done", C.c_int64), ("kernels_per_pass", C.c_int32),
                ("n_stages", C.c_int32), ("r2", C.c_double), ("stage_ms", C.c_double * 16),
                ("stage_calls", C.c_int64 * 16), ("candidates", C.c_int64), ("in_radius", C.c_int64),
                ("gather_slots", C.c_int64), ("cell_factor", C.c_int32), ("photon_rays", C.c_int64),
                ("eye_rays", C.c_int64)]


class GatherExport(C.Structure):
    """ppm_gather_export (include/ppm_api.h): the render gather's per-hit-point parity export."""
    _fields_ = [("photon_cap", C.c_int64), ("hit_cap", C.c_int64), ("n_photons", C.c_int64), ("n_hits", C.c_int64),
                ("radius2", C.c_double), ("photon_power", C.c_double), ("pass_", C.c_int32), ("pfilter", C.c_int32),
                ("photons", C.POINTER(C.c_float)), ("hits", C.POINTER(C.c_float)), ("sums", C.POINTER(C.c_float)),
                ("counts", C.POINTER(C.c_uint32)), ("checksums", C.POINTER(C.c_uint64)),
                ("gathered", C.POINTER(C.c_float))]


# ---------------------------------------------------------------------------
# vector helpers in the reference's evaluation order (src/ray/algebra.rs)
# ---------------------------------------------------------------------------
def _sub(a, b):
    return (a[0] - b[0], a[1] - b[1], a[2] - b[2])


def _cross(a, b):
    return (a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1])


def _dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def normalize(v):
    """Vector3::normalize (algebra.rs:186-194): v * (1/|v|), None for zero."""
    n = math.sqrt(_dot(v, v))
    if n == 0.0:
        return None
    r = 1.0 / n
    return (v[0] * r, v[1] * r, v[2] * r)


def color_normalize(c):
    """Color::normalize (physics.rs:61-71)."""
    r1, g1, b1 = (x if x >= 0.0 else 0.0 for x in c)
    mag = r1 + g1 + b1
    if mag == 0.0:
        return (1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0)
    return (r1 / mag, g1 / mag, b1 / mag)


# ---------------------------------------------------------------------------
# shapes (src/ray/geometry.rs:66-115)
# ---------------------------------------------------------------------------
@dataclass
class Shape:
    shape: int
    position: tuple = (0.0, 0.0, 0.0)
    nvec: tuple = (0.0, 0.0, 0.0)
    dir1: tuple = (0.0, 0.0, 0.0)
    dir2: tuple = (0.0, 0.0, 0.0)
    dist: float = 0.0
    radius: float = 0.0


def plain(nvec, dist) -> Shape:
    """Shape::Plain: the infinite plane nvec . x + dist = 0."""
    return Shape(SHAPE_PLAIN, nvec=tuple(map(float, nvec)), dist=float(dist))


def sphere(center, radius) -> Shape:
    return Shape(SHAPE_SPHERE, position=tuple(map(float, center)), radius=float(radius))


def polygon(p0, p1, p2) -> Shape:
    """Shape::new_polygon (geometry.rs:93-103)."""
    d1, d2 = _sub(p1, p0), _sub(p2, p0)
    return Shape(SHAPE_POLYGON, position=tuple(map(float, p0)), nvec=normalize(_cross(d1, d2)), dir1=d1, dir2=d2)


def parallelogram(p0, p1, p2) -> Shape:
    """Shape::new_parallelogram (geometry.rs:105-115)."""
    d1, d2 = _sub(p1, p0), _sub(p2, p0)
    return Shape(SHAPE_PARALLELOGRAM, position=tuple(map(float, p0)), nvec=normalize(_cross(d1, d2)), dir1=d1, dir2=d2)


def parallelogram_raw(position, nvec, dir1, dir2) -> Shape:
    """Shape::Parallelogram with explicit fields (as src/scene.rs:424-430 writes it)."""
    return Shape(SHAPE_PARALLELOGRAM, position=tuple(map(float, position)), nvec=tuple(map(float, nvec)),
                 dir1=tuple(map(float, dir1)), dir2=tuple(map(float, dir2)))


# ---------------------------------------------------------------------------
# materials (src/ray/surface.rs:45-66, material.rs:11-16)
# ---------------------------------------------------------------------------
@dataclass
class Mat:
    surface: int
    color_diff: tuple
    color_spec: tuple
    scatter: float
    metalness: float
    roughness: float
    emittance: tuple = (0.0, 0.0, 0.0)
    transmittance: tuple = (0.0, 0.0, 0.0)
    ior: tuple = (0.0, 0.0, 0.0)

    @property
    def density_pow(self) -> float:
        return 1.0 / (10.0 ** (5.0 * (1.0 - math.sqrt(self.roughness))) + 1.0)

    @property
    def alpha(self) -> float:
        r = self.roughness
        return r * r * r * r if self.surface == SURF_TS else 0.0


def new_simple(refl, spec, diff, meta, rough, *, emittance=(0.0, 0.0, 0.0), transmittance=(0.0, 0.0, 0.0),
               ior=(0.0, 0.0, 0.0)) -> Mat:
    """Material with Surface::new_simple(reflectance, specular_refl, diffuseness, metalness, roughness)."""
    return Mat(SURF_SIMPLE, tuple(map(float, refl)), tuple(map(float, spec)), float(diff), float(meta), float(rough),
               tuple(map(float, emittance)), tuple(map(float, transmittance)), tuple(map(float, ior)))


def new_ts(al_diff, al_spec, scat, meta, rough, *, emittance=(0.0, 0.0, 0.0), transmittance=(0.0, 0.0, 0.0),
           ior=(0.0, 0.0, 0.0)) -> Mat:
    """Material with Surface::new_ts(albedo_diff, albedo_spec, scatterness, metalness, roughness)."""
    return Mat(SURF_TS, tuple(map(float, al_diff)), tuple(map(float, al_spec)), float(scat), float(meta), float(rough),
               tuple(map(float, emittance)), tuple(map(float, transmittance)), tuple(map(float, ior)))


# ---------------------------------------------------------------------------
# lights (src/ray/light.rs:16-39)
# ---------------------------------------------------------------------------
@dataclass
class Lgt:
    kind: int
    color: tuple
    flux: float
    pos: tuple
    nvec: tuple = (0.0, 0.0, 0.0)
    dir1: tuple = (0.0, 0.0, 0.0)
    dir2: tuple = (0.0, 0.0, 0.0)
    dir: tuple = (0.0, 0.0, 0.0)


def point_light(color, flux, pos) -> Lgt:
    return Lgt(LIGHT_POINT, tuple(map(float, color)), float(flux), tuple(map(float, pos)))


def parallelogram_light(color, flux, pos, nvec, dir1, dir2) -> Lgt:
    return Lgt(LIGHT_PARALLELOGRAM, tuple(map(float, color)), float(flux), tuple(map(float, pos)),
               tuple(map(float, nvec)), tuple(map(float, dir1)), tuple(map(float, dir2)))


def spot_light(color, flux, pos, axis, half_angle_deg) -> Lgt:
    """Spot light (no reference counterpart): a point light emitting only into
    the cone of the given half-angle around axis; the C ABI carries the unit
    axis in dir and cos(half-angle) in dir1[0]."""
    a = normalize(tuple(map(float, axis)))
    cc = math.cos(math.radians(float(half_angle_deg)))
    return Lgt(LIGHT_SPOT, tuple(map(float, color)), float(flux), tuple(map(float, pos)), (0.0, 0.0, 0.0),
               (cc, 0.0, 0.0), (0.0, 0.0, 0.0), a)


def sun_light(color, flux, pos, nvec, dir1, dir2, direction) -> Lgt:
    return Lgt(LIGHT_SUN, tuple(map(float, color)), float(flux), tuple(map(float, pos)), tuple(map(float, nvec)),
               tuple(map(float, dir1)), tuple(map(float, dir2)), tuple(map(float, direction)))


# ---------------------------------------------------------------------------
# scene container
# ---------------------------------------------------------------------------
def _object_dtype():
    """numpy view of ppm_object (120 bytes)."""
    import numpy as np
    return np.dtype({"names": ["shape", "material", "position", "nvec", "dir1", "dir2", "dist", "radius"],
                     "formats": ["<i4", "<i4", ("<f8", 3), ("<f8", 3), ("<f8", 3), ("<f8", 3), "<f8", "<f8"],
                     "offsets": [0, 4, 8, 32, 56, 80, 104, 112], "itemsize": C.sizeof(Object)})


@dataclass
class Scene:
    objects: List[tuple] = field(default_factory=list)   # (Shape, material index)
    materials: List[Mat] = field(default_factory=list)
    lights: List[Lgt] = field(default_factory=list)
    # objects added in bulk (numpy rows of the ppm_object layout), after `objects`
    bulk: list = field(default_factory=list)

    def _bulk_rows(self, n, shape, mats):
        import numpy as np
        rows = np.zeros(n, _object_dtype())
        rows["shape"] = shape
        rows["material"] = np.broadcast_to(np.asarray(mats, np.int32), (n,))
        self.bulk.append(rows)
        return rows

    def _bulk_flat(self, shape, p0, p1, p2, mats):
        import numpy as np
        p0 = np.ascontiguousarray(p0, np.float64)
        d1 = np.ascontiguousarray(p1, np.float64) - p0
        d2 = np.ascontiguousarray(p2, np.float64) - p0
        n = np.cross(d1, d2)
        n /= np.linalg.norm(n, axis=1, keepdims=True)
        r = self._bulk_rows(len(p0), shape, mats)
        r["position"], r["nvec"], r["dir1"], r["dir2"] = p0, n, d1, d2

    def add_triangles(self, p0, p1, p2, mats):
        """Triangles p0 p1 p2 (n x 3 each, counter-clockwise seen from the
        normal's side) as Shape::new_polygon builds them (geometry.rs:93-103):
        dir1 = p1 - p0, dir2 = p2 - p0, nvec = normalize(dir1 x dir2)."""
        self._bulk_flat(SHAPE_POLYGON, p0, p1, p2, mats)

    def add_parallelograms(self, p0, p1, p2, mats):
        """Shape::new_parallelogram (geometry.rs:105-115) for n x 3 corner arrays."""
        self._bulk_flat(SHAPE_PARALLELOGRAM, p0, p1, p2, mats)

    def add_spheres(self, centres, radii, mats):
        import numpy as np
        c = np.ascontiguousarray(centres, np.float64)
        r = self._bulk_rows(len(c), SHAPE_SPHERE, mats)
        r["position"], r["radius"] = c, np.broadcast_to(np.asarray(radii, np.float64), (len(c),))

    @property
    def n_objects(self) -> int:
        return len(self.objects) + sum(len(b) for b in self.bulk)

    def add_material(self, m: Mat) -> int:
        self.materials.append(m)
        return len(self.materials) - 1

    def add(self, shape: Shape, mat: int) -> int:
        self.objects.append((shape, mat))
        return len(self.objects) - 1

    def c_objects(self):
        n = self.n_objects
        arr = (Object * max(1, n))()
        for i, (s, m) in enumerate(self.objects):
            o = arr[i]
            o.shape, o.material = s.shape, m
            o.position[:], o.nvec[:], o.dir1[:], o.dir2[:] = s.position, s.nvec, s.dir1, s.dir2
            o.dist, o.radius = s.dist, s.radius
        if self.bulk:
            import numpy as np
            view = np.frombuffer(arr, dtype=_object_dtype())
            k = len(self.objects)
            for b in self.bulk:
                view[k:k + len(b)] = b
                k += len(b)
        return arr, n

    def c_materials(self):
        arr = (Material * max(1, len(self.materials)))()
        for i, m in enumerate(self.materials):
            c = arr[i]
            c.emittance[:], c.transmittance[:], c.ior[:] = m.emittance, m.transmittance, m.ior
            c.surface = m.surface
            c.color_diff[:], c.color_spec[:] = m.color_diff, m.color_spec
            c.scatter, c.metalness, c.roughness = m.scatter, m.metalness, m.roughness
            c.density_pow, c.alpha = m.density_pow, m.alpha
        return arr, len(self.materials)

    def c_lights(self):
        arr = (Light * max(1, len(self.lights)))()
        for i, l in enumerate(self.lights):
            c = arr[i]
            c.kind, c.flux = l.kind, l.flux
            c.color[:], c.pos[:], c.nvec[:], c.dir1[:], c.dir2[:], c.dir[:] = (
                l.color, l.pos, l.nvec, l.dir1, l.dir2, l.dir)
        return arr, len(self.lights)


# ---------------------------------------------------------------------------
# camera (src/camera.rs:108-206)
# ---------------------------------------------------------------------------
def make_camera(xreso=256, yreso=256, *, progressive=True, antialias=True, use_classic=True, blur=True,
                estimate_radius=0.2, max_radiance=0.01, iso_sensitivity=100.0, shutter_speed=0.004,
                focal_length_mm=50.0, f_number=4.0, focus=7.0, photon_filter=FILTER_NONE,
                ambient=(0.0, 0.0, 0.0), eye_position=(1.0, 2.0, -4.5), target_position=(0.0, 1.0, 0.0),
                upper_direction=(0.0, 1.0, 0.0)) -> Camera:
    """read_camera's parameter map (camera.rs:108-146); defaults are the reference's.
    The derived fields are filled by camera_derive (or by ppm_camera_set)."""
    c = Camera()
    c.xreso, c.yreso = int(xreso), int(yreso)
    c.progressive, c.antialias, c.use_classic, c.blur = int(progressive), int(antialias), int(use_classic), int(blur)
    c.pfilter, c.n_sample_photon = int(photon_filter), 500
    c.radius = estimate_radius * estimate_radius
    c.max_radiance, c.iso_sens, c.shut_speed = max_radiance, iso_sensitivity, shutter_speed
    c.focal_len = focal_length_mm / 1000.0
    c.f_number, c.focus = f_number, focus
    c.ambient[:], c.eye_pos[:], c.target[:], c.upper[:] = ambient, eye_position, target_position, upper_direction
    camera_derive(c)
    return c


def camera_derive(c: Camera) -> None:
    """The derived block of read_camera (camera.rs:150-175), in the same order."""
    SENSOR, ISO, FNUM, SHUT = 35.0 / 1000.0, 100.0, 4.9, 1.0 / 250.0
    eye, tgt, up = tuple(c.eye_pos), tuple(c.target), tuple(c.upper)
    ez = normalize(_sub(tgt, eye))
    ex = normalize(_cross(up, ez))
    ey = normalize(_cross(ex, ez))
    step = (c.focus * SENSOR / c.focal_len) / float(c.xreso)
    sm = lambda s, v: (s * v[0], s * v[1], s * v[2])  # noqa: E731
    esx, esy = sm(step, ex), sm(step, ey)
    ea = c.focal_len / c.f_number
    eex, eey = sm(ea, ex), sm(ea, ey)
    lx, ly = float(c.xreso // 2), float(c.yreso // 2)
    orig = _sub(_sub(sm(c.focus, ez), sm(lx - 0.5, esx)), sm(ly - 0.5, esy))
    c.photon_power = (c.iso_sens / ISO * FNUM / c.f_number * c.shut_speed / SHUT) if c.blur else 1.0
    c.eye_dir[:] = normalize(_sub(tgt, eye))
    c.origin[:], c.esx[:], c.esy[:], c.eex[:], c.eey[:] = orig, esx, esy, eex, eey


# ---------------------------------------------------------------------------
# scenes
# ---------------------------------------------------------------------------
def reference_scene() -> Scene:
    """The scene that read_scene returns (src/scene.rs:20-448), restated as data."""
    sc = Scene()
    sc.lights.append(parallelogram_light(color_normalize((1.0, 1.0, 1.0)), 5.0, (-0.67, 3.99, 2.33),
                                         (-0.0, -1.0, -0.0), (1.33, 0.0, 0.0), (0.0, 0.0, 1.33)))
    mwall = sc.add_material(new_simple((0.5, 0.5, 0.5), (0.8, 0.8, 0.8), 1.0, 0.0, 0.0))
    mwallb = sc.add_material(new_simple((0.1, 0.1, 0.4), (0.8, 0.0, 0.8), 1.0, 0.0, 0.0))
    mwallr = sc.add_material(new_simple((0.4, 0.1, 0.1), (0.0, 0.0, 0.0), 1.0, 0.0, 0.0))
    ball10 = sc.add_material(new_ts((1.0, 1.0, 1.0), (0.05, 0.05, 0.05), 0.0, 0.0, 0.8, ior=(1.5, 1.5, 1.5)))
    ball9 = sc.add_material(new_simple((0.0, 0.0, 0.0), (0.78, 0.78, 0.78), 0.0, 1.0, 0.9))
    ball8 = sc.add_material(new_simple((0.0, 0.0, 0.0), (0.78, 0.78, 0.78), 0.0, 1.0, 0.8))
    ball7 = sc.add_material(new_simple((0.0, 0.0, 0.0), (0.78, 0.78, 0.78), 0.0, 1.0, 0.7))
    ball6 = sc.add_material(new_ts((0.0, 0.0, 0.0), (0.78, 0.78, 0.78), 0.0, 1.0, 0.6))
    ball5 = sc.add_material(new_ts((0.0, 0.0, 0.0), (0.78, 0.78, 0.78), 0.0, 1.0, 0.5))
    ball4 = sc.add_material(new_simple((0.0, 0.0, 0.0), (0.78, 0.78, 0.78), 0.0, 1.0, 0.4))
    ball3 = sc.add_material(new_simple((0.0, 0.0, 0.0), (0.78, 0.78, 0.78), 0.0, 1.0, 0.3))
    ball2 = sc.add_material(new_simple((0.0, 0.0, 0.0), (0.78, 0.78, 0.78), 0.0, 1.0, 0.2))
    ball1 = sc.add_material(new_ts((0.6, 0.35, 0.1), (0.05, 0.05, 0.05), 1.0, 0.0, 0.0, ior=(1.5, 1.5, 1.5)))
    mparal = sc.add_material(new_simple((0.0, 0.0, 0.0), (0.8, 0.8, 0.8), 0.0, 0.0, 0.0,
                                        emittance=(0.15, 0.15, 0.15)))
    sc.add(plain((0.0, 1.0, 0.0), 0.0), mwall)        # flooring
    sc.add(plain((-0.0, -1.0, -0.0), 4.0), mwall)     # ceiling
    sc.add(plain((-1.0, -0.0, -0.0), 2.0), mwallb)    # right side wall
    sc.add(plain((1.0, 0.0, 0.0), 2.0), mwallr)       # left side wall
    sc.add(plain((0.0, 0.0, 1.0), 6.0), mwall)        # back wall
    sc.add(plain((-0.0, -0.0, -1.0), 5.0), mwall)     # front wall
    for cx, m in ((-1.6, ball1), (-0.8, ball2), (0.0, ball3), (0.8, ball4), (1.6, ball5)):
        sc.add(sphere((cx, 1.5, 3.0), 0.4), m)
    for cx, m in ((-1.6, ball6), (-0.8, ball7), (0.0, ball8), (0.8, ball9), (1.6, ball10)):
        sc.add(sphere((cx, 0.5, 2.5), 0.4), m)
    sc.add(parallelogram_raw((-0.67, 3.99, 2.33), (-0.0, -1.0, -0.0),
                             _sub((0.67, 3.99, 2.33), (-0.67, 3.99, 2.33)),
                             _sub((-0.67, 3.99, 3.67), (-0.67, 3.99, 2.33))), mparal)
    return sc


def reference_camera() -> Camera:
    """The camera that read_camera returns (src/camera.rs:108-206)."""
    return make_camera()


def box_scene(variant: str = "c1") -> Scene:
    """Closed box of five diffuse quads (open towards the camera) with a point
    light below the ceiling.  c1: one diffuse sphere (reflectance 0.75) and
    one mirror sphere; c2: the diffuse sphere replaced by glass (TS, IOR 1.5).
    Box x in [-1, 1], y in [0, 2], z in [0, 2]; spheres r = 0.3."""
    sc = Scene()
    white = sc.add_material(new_simple((0.75, 0.75, 0.75), (0.0, 0.0, 0.0), 1.0, 0.0, 0.0))
    red = sc.add_material(new_simple((0.75, 0.0, 0.0), (0.0, 0.0, 0.0), 1.0, 0.0, 0.0))
    green = sc.add_material(new_simple((0.0, 0.75, 0.0), (0.0, 0.0, 0.0), 1.0, 0.0, 0.0))
    mirror = sc.add_material(new_simple((0.0, 0.0, 0.0), (0.78, 0.78, 0.78), 0.0, 1.0, 0.0))
    if variant == "c1":
        ball = sc.add_material(new_simple((0.75, 0.75, 0.75), (0.0, 0.0, 0.0), 1.0, 0.0, 0.0))
    elif variant == "c2":
        ball = sc.add_material(new_ts((1.0, 1.0, 1.0), (0.05, 0.05, 0.05), 0.0, 0.0, 0.0, ior=(1.5, 1.5, 1.5)))
    else:
        raise ValueError(f"unknown box variant {variant!r}")
    sc.add(parallelogram((-1.0, 0.0, 2.0), (1.0, 0.0, 2.0), (-1.0, 2.0, 2.0)), white)   # back
    sc.add(parallelogram((-1.0, 0.0, 0.0), (-1.0, 0.0, 2.0), (1.0, 0.0, 0.0)), white)   # floor
    sc.add(parallelogram((-1.0, 2.0, 0.0), (1.0, 2.0, 0.0), (-1.0, 2.0, 2.0)), white)   # ceiling
    sc.add(parallelogram((-1.0, 0.0, 0.0), (-1.0, 2.0, 0.0), (-1.0, 0.0, 2.0)), red)    # left
    sc.add(parallelogram((1.0, 0.0, 0.0), (1.0, 0.0, 2.0), (1.0, 2.0, 0.0)), green)     # right
    sc.add(sphere((-0.45, 0.3, 1.2), 0.3), ball)
    sc.add(sphere((0.45, 0.3, 0.9), 0.3), mirror)
    sc.lights.append(point_light(color_normalize((1.0, 1.0, 1.0)), 100.0, (0.0, 1.95, 1.0)))
    return sc


def box_camera(reso: int = 256) -> Camera:
    """Pinhole view into the box (no lens blur); anti-aliasing jitter per pass."""
    return make_camera(reso, reso, progressive=True, antialias=True, use_classic=True, blur=False,
                       eye_position=(0.0, 1.0, -2.6), target_position=(0.0, 1.0, 1.0), focus=3.6)

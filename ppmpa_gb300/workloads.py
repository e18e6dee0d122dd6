"""Seeded synthetic inputs for the FP32 photon-map gather sweep.

Photons: FP32 positions, unit directions, one wavelength each, drawn either
uniform in the unit cube or clustered (90 % in 1000 Gaussian caustic blobs of
sigma 0.002 with centres uniform in the cube, 10 % uniform).  Queries: FP32
positions from the same distribution (same blob centres), unit normals
uniform on the sphere, radii log-uniform over [1e-3, 2e-2].

Arrays are generated in chunks so that 100M photons need no more than the
outputs plus one chunk of temporaries.
"""
import numpy as np

R_MIN, R_MAX = 1e-3, 2e-2
N_BLOBS, BLOB_SIGMA, BLOB_FRACTION = 1000, 0.002, 0.9
PHOTON_SEED, QUERY_SEED = 42, 43
CHUNK = 1 << 22


def _centres(seed):
    return np.random.default_rng([seed, 7]).random((N_BLOBS, 3)).astype(np.float32)


def _positions(rng, n, kind, centres, out):
    if kind == "uniform":
        for a in range(0, n, CHUNK):
            b = min(n, a + CHUNK)
            out[a:b] = rng.random((b - a, 3), dtype=np.float32)
        return
    if kind != "clustered":
        raise ValueError(f"unknown photon distribution {kind!r}")
    for a in range(0, n, CHUNK):
        b = min(n, a + CHUNK)
        m = b - a
        in_blob = rng.random(m) < BLOB_FRACTION
        which = rng.integers(0, N_BLOBS, m)
        p = centres[which] + np.float32(BLOB_SIGMA) * rng.standard_normal((m, 3), dtype=np.float32)
        u = rng.random((m, 3), dtype=np.float32)
        out[a:b] = np.where(in_blob[:, None], p, u)


def _unit(rng, n, out):
    for a in range(0, n, CHUNK):
        b = min(n, a + CHUNK)
        v = rng.standard_normal((b - a, 3), dtype=np.float32)
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        out[a:b] = v


def photons(n: int, kind: str = "uniform", seed: int = PHOTON_SEED):
    """(pos f32 n x 3, dir f32 n x 3, wl u8 n)."""
    rng = np.random.default_rng(seed)
    pos = np.empty((n, 3), np.float32)
    _positions(rng, n, kind, _centres(seed), pos)
    d = np.empty((n, 3), np.float32)
    _unit(rng, n, d)
    wl = rng.integers(0, 3, n, dtype=np.uint8)
    return pos, d, wl


def queries(n: int, kind: str = "uniform", seed: int = QUERY_SEED, photon_seed: int = PHOTON_SEED):
    """(pos f32 n x 3, normal f32 n x 3, r2 f64 n) with r log-uniform in [R_MIN, R_MAX]."""
    rng = np.random.default_rng(seed)
    pos = np.empty((n, 3), np.float32)
    _positions(rng, n, kind, _centres(photon_seed), pos)
    nrm = np.empty((n, 3), np.float32)
    _unit(rng, n, nrm)
    r = np.exp(rng.uniform(np.log(R_MIN), np.log(R_MAX), n))
    return pos, nrm, r * r


def oct_roundtrip(d):
    """Directions as the FP32 map stores them: octahedral 15+15-bit codes,
    decoded and renormalised in FP64 (the oracle's view of the map)."""
    d = np.asarray(d, np.float32)
    a = np.abs(d)
    s = (a[:, 0] + a[:, 1]) + a[:, 2]
    inv = np.float32(1) / s                    # the encoder multiplies by 1/s, as here
    p = d[:, :2] * inv[:, None]
    neg = d[:, 2] < 0
    sg = np.where(p >= 0, np.float32(1), np.float32(-1))
    fold = (np.float32(1) - np.abs(p[:, ::-1])) * sg
    p = np.where(neg[:, None], fold, p)
    qv = np.clip(np.rint((p * np.float32(0.5) + np.float32(0.5)) * np.float32(32767)), 0, 32767)
    p = qv.astype(np.float32) * np.float32(2.0 / 32767.0) - np.float32(1)
    z = np.float32(1) - np.abs(p[:, 0]) - np.abs(p[:, 1])
    sg = np.where(p >= 0, np.float32(1), np.float32(-1))
    fold = (np.float32(1) - np.abs(p[:, ::-1])) * sg
    p = np.where((z < 0)[:, None], fold, p)
    v = np.column_stack([p, z]).astype(np.float64)
    return v / np.linalg.norm(v, axis=1, keepdims=True)


# ---------------------------------------------------------------------------
# batch of uneven render jobs
# ---------------------------------------------------------------------------
def _log_uniform(rng, lo, hi):
    return float(np.exp(rng.uniform(np.log(lo), np.log(hi))))


def batch_scene(rng, n_prims: int):
    """The closed box with n_prims spheres and quads (half each) inside,
    materials drawn from diffuse / mirror / glass, one point or one
    parallelogram light under the ceiling."""
    from . import scene as S
    sc = S.Scene()
    white = sc.add_material(S.new_simple((0.75, 0.75, 0.75), (0.0, 0.0, 0.0), 1.0, 0.0, 0.0))
    red = sc.add_material(S.new_simple((0.75, 0.0, 0.0), (0.0, 0.0, 0.0), 1.0, 0.0, 0.0))
    green = sc.add_material(S.new_simple((0.0, 0.75, 0.0), (0.0, 0.0, 0.0), 1.0, 0.0, 0.0))
    mirror = sc.add_material(S.new_simple((0.0, 0.0, 0.0), (0.78, 0.78, 0.78), 0.0, 1.0, 0.0))
    glass = sc.add_material(S.new_ts((1.0, 1.0, 1.0), (0.05, 0.05, 0.05), 0.0, 0.0, 0.0, ior=(1.5, 1.5, 1.5)))
    sc.add(S.parallelogram((-1.0, 0.0, 2.0), (1.0, 0.0, 2.0), (-1.0, 2.0, 2.0)), white)
    sc.add(S.parallelogram((-1.0, 0.0, 0.0), (-1.0, 0.0, 2.0), (1.0, 0.0, 0.0)), white)
    sc.add(S.parallelogram((-1.0, 2.0, 0.0), (1.0, 2.0, 0.0), (-1.0, 2.0, 2.0)), white)
    sc.add(S.parallelogram((-1.0, 0.0, 0.0), (-1.0, 2.0, 0.0), (-1.0, 0.0, 2.0)), red)
    sc.add(S.parallelogram((1.0, 0.0, 0.0), (1.0, 0.0, 2.0), (1.0, 2.0, 0.0)), green)
    palette = np.array([white, white, red, green, mirror, glass], np.int32)
    n_s = n_prims // 2
    n_q = n_prims - n_s
    size = 0.35 * (6.0 / max(1, n_prims)) ** (1.0 / 3.0)       # fills a fraction of the box
    lo, hi = np.array([-0.9, 0.1, 0.1]), np.array([0.9, 1.8, 1.9])
    if n_s:
        c = rng.uniform(lo, hi, (n_s, 3))
        sc.add_spheres(c, size * rng.uniform(0.5, 1.0, n_s), palette[rng.integers(0, len(palette), n_s)])
    if n_q:
        p0 = rng.uniform(lo, hi, (n_q, 3))
        a = rng.normal(size=(n_q, 3))
        b = rng.normal(size=(n_q, 3))
        a *= size / np.linalg.norm(a, axis=1, keepdims=True)
        b *= size / np.linalg.norm(b, axis=1, keepdims=True)
        sc.add_parallelograms(p0, p0 + a, p0 + b, palette[rng.integers(0, len(palette), n_q)])
    col = S.color_normalize((1.0, 1.0, 1.0))
    if rng.random() < 0.5:
        sc.lights.append(S.point_light(col, 100.0, (0.0, 1.95, 1.0)))
    else:
        sc.lights.append(S.parallelogram_light(col, 100.0, (-0.3, 1.99, 0.7), (0.0, -1.0, 0.0), (0.6, 0.0, 0.0),
                                               (0.0, 0.0, 0.6)))
    return sc


def batch_jobs(n_jobs: int = 64, seed: int = 7, passes: int = 8, precision: int = 1, flags: int = 1,
               prims=(10, 200_000), reso=(64, 512), photons=(50_000, 2_000_000)):
    """[(scene, camera, RenderConfig)]: primitive counts log-uniform over
    `prims`, square images `reso` pixels wide (log-uniform), photons per
    pass log-uniform over `photons`, alpha uniform in [0.5, 0.9]."""
    from . import scene as S
    from .api import RenderConfig
    rng = np.random.default_rng([seed, 404])
    jobs = []
    for j in range(n_jobs):
        n_prims = int(round(_log_uniform(rng, *prims)))
        w = int(round(_log_uniform(rng, *reso)))
        nphoton = int(round(_log_uniform(rng, *photons)))
        alpha = float(rng.uniform(0.5, 0.9))
        sc = batch_scene(rng, n_prims)
        cfg = RenderConfig(nphoton=nphoton, passes=passes, radius0=0.05, alpha=alpha, precision=precision,
                           seed=seed * 1000 + j, flags=flags)
        jobs.append((sc, S.box_camera(w), cfg))
    return jobs

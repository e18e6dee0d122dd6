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

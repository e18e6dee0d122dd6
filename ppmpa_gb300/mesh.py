"""Seeded triangle meshes for the large-mesh workload.

icosphere(level): the icosahedron with every face split into four `level`
times, vertices pushed to the unit sphere (20 * 4**level faces; level 8 =
1,310,720).  Faces are counter-clockwise seen from outside, so the normals
Shape::new_polygon derives point outwards and a closed glass mesh tracks
inside/outside like the reference's spheres.

perlin(points, seed): gradient noise after K. Perlin, "Improving noise"
(SIGGRAPH 2002) -- quintic fade, 12 edge gradients picked by a hash of the
lattice cell -- with the permutation table shuffled by `seed`.

mesh_scene(): the closed box of the box scenes with a displaced icosphere
(radial displacement by 3-octave noise, amplitude 5 % of the radius), half
its faces glass and half diffuse by a seeded mask, lit by a spot light below
the ceiling.
"""
import math

import numpy as np

from . import scene as S

_ICO_FACES = np.array([
    (0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
    (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
    (8, 6, 7), (9, 8, 1)], np.int64)


def _ico_vertices():
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
                  (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], np.float64)
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def icosphere(level: int):
    """(vertices V x 3 on the unit sphere, faces F x 3 int64, outward CCW)."""
    v = _ico_vertices()
    f = _ICO_FACES.copy()
    # orient every face outwards
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    flip = np.einsum("ij,ij->i", n, v[f].sum(1)) < 0
    f[flip] = f[flip][:, ::-1]
    for _ in range(level):
        nv = len(v)
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        key = np.minimum(e[:, 0], e[:, 1]) * nv + np.maximum(e[:, 0], e[:, 1])
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = uniq // nv, uniq % nv
        mid = v[a] + v[b]
        v = np.concatenate([v, mid / np.linalg.norm(mid, axis=1, keepdims=True)])
        m = nv + inv.reshape(3, -1)          # midpoints of edges 01, 12, 20 per face
        ab, bc, ca = m[0], m[1], m[2]
        f = np.concatenate([np.stack([f[:, 0], ab, ca], 1), np.stack([f[:, 1], bc, ab], 1),
                            np.stack([f[:, 2], ca, bc], 1), np.stack([ab, bc, ca], 1)])
    return v, f


def _perm(seed):
    p = np.random.default_rng([seed, 101]).permutation(256)
    return np.concatenate([p, p])


def _fade(t):
    return t * t * t * (t * (t * 6.0 - 15.0) + 10.0)


def _grad(h, x, y, z):
    h = h & 15
    u = np.where(h < 8, x, y)
    v = np.where(h < 4, y, np.where((h == 12) | (h == 14), x, z))
    return np.where(h & 1, -u, u) + np.where(h & 2, -v, v)


def perlin(p, seed: int = 1):
    """Noise in about [-1, 1] at points p (n x 3)."""
    perm = _perm(seed)
    fl = np.floor(p)
    c = fl.astype(np.int64) & 255
    x, y, z = (p - fl).T
    u, v, w = _fade(x), _fade(y), _fade(z)
    X, Y, Z = c.T
    A = perm[X] + Y
    AA, AB = perm[A] + Z, perm[A + 1] + Z
    B = perm[X + 1] + Y
    BA, BB = perm[B] + Z, perm[B + 1] + Z
    lerp = lambda t, a, b: a + t * (b - a)
    return lerp(w,
                lerp(v, lerp(u, _grad(perm[AA], x, y, z), _grad(perm[BA], x - 1, y, z)),
                     lerp(u, _grad(perm[AB], x, y - 1, z), _grad(perm[BB], x - 1, y - 1, z))),
                lerp(v, lerp(u, _grad(perm[AA + 1], x, y, z - 1), _grad(perm[BA + 1], x - 1, y, z - 1)),
                     lerp(u, _grad(perm[AB + 1], x, y - 1, z - 1), _grad(perm[BB + 1], x - 1, y - 1, z - 1))))


def displaced_icosphere(level: int, centre, radius: float, amplitude: float = 0.05, frequency: float = 3.0,
                        octaves: int = 3, seed: int = 1):
    """Vertices displaced radially by amplitude * radius * fBm noise."""
    v, f = icosphere(level)
    n = np.zeros(len(v))
    norm = 0.0
    for o in range(octaves):
        n += 0.5 ** o * perlin(v * (frequency * 2 ** o) + 17.0, seed + o)
        norm += 0.5 ** o
    n /= norm
    r = radius * (1.0 + amplitude * np.clip(n, -1.0, 1.0))
    return v * r[:, None] + np.asarray(centre, np.float64), f


def mesh_scene(level: int = 8, seed: int = 1, spot_half_angle: float = 35.0) -> S.Scene:
    """Box (x in [-1, 1], y and z in [0, 2]) + displaced icosphere (centre
    (0, 0.75, 1), radius 0.55), faces glass (TS, IOR 1.5) or diffuse white by
    a seeded 50 % mask, spot light 100 W at (0, 1.95, 1) pointing down."""
    sc = S.Scene()
    white = sc.add_material(S.new_simple((0.75, 0.75, 0.75), (0.0, 0.0, 0.0), 1.0, 0.0, 0.0))
    red = sc.add_material(S.new_simple((0.75, 0.0, 0.0), (0.0, 0.0, 0.0), 1.0, 0.0, 0.0))
    green = sc.add_material(S.new_simple((0.0, 0.75, 0.0), (0.0, 0.0, 0.0), 1.0, 0.0, 0.0))
    glass = sc.add_material(S.new_ts((1.0, 1.0, 1.0), (0.05, 0.05, 0.05), 0.0, 0.0, 0.0, ior=(1.5, 1.5, 1.5)))
    diffuse = sc.add_material(S.new_simple((0.75, 0.75, 0.75), (0.0, 0.0, 0.0), 1.0, 0.0, 0.0))
    sc.add(S.parallelogram((-1.0, 0.0, 2.0), (1.0, 0.0, 2.0), (-1.0, 2.0, 2.0)), white)   # back
    sc.add(S.parallelogram((-1.0, 0.0, 0.0), (-1.0, 0.0, 2.0), (1.0, 0.0, 0.0)), white)   # floor
    sc.add(S.parallelogram((-1.0, 2.0, 0.0), (1.0, 2.0, 0.0), (-1.0, 2.0, 2.0)), white)   # ceiling
    sc.add(S.parallelogram((-1.0, 0.0, 0.0), (-1.0, 2.0, 0.0), (-1.0, 0.0, 2.0)), red)    # left
    sc.add(S.parallelogram((1.0, 0.0, 0.0), (1.0, 0.0, 2.0), (1.0, 2.0, 0.0)), green)     # right
    v, f = displaced_icosphere(level, (0.0, 0.75, 1.0), 0.55, seed=seed)
    mask = np.random.default_rng([seed, 202]).random(len(f)) < 0.5
    sc.add_triangles(v[f[:, 0]], v[f[:, 1]], v[f[:, 2]], np.where(mask, glass, diffuse))
    sc.lights.append(S.spot_light(S.color_normalize((1.0, 1.0, 1.0)), 100.0, (0.0, 1.95, 1.0), (0.0, -1.0, 0.0),
                                  spot_half_angle))
    return sc

"""Conservativeness of the FP32 photon-map grid, on the CPU: a float32
restatement of the grid set-up (k_grid_setup), the cell coordinates
(CellMath<float>), the query's cell ranges (query_cells) and the row
culling (RowCull<float>::range) checks that the rows and x-ranges the
gather walks hold every photon within the radius -- for single queries and
for the union the paired walk takes over two queries of one cell -- with
queries and photons placed on and around cell boundaries.  (The GPU may
contract some of these products into FMAs; the margins the test exercises
are the ones that absorb such rounding.)"""
import numpy as np
import pytest

f32 = np.float32


def grid(lo, hi, r2, k=1.0, sx=4, cell_cap=1 << 24):
    r = np.sqrt(r2)
    c = r * ((1.0 + 1.0 / 128.0) / k)
    inv = 1.0 / c
    while True:
        dim = [int(np.floor((hi[a] - lo[a]) * (inv * sx if a == 0 else inv))) + 1 for a in range(3)]
        if all(d <= 8192 for d in dim) and dim[0] * dim[1] * dim[2] <= cell_cap:
            break
        c *= 1.25
        inv = 1.0 / c
    invx = inv * sx
    ext = int(min(max(np.ceil(r * inv + 3e-3), 1), 8))
    extx = int(min(max(np.ceil(r * invx + 3e-3), 1), 64))
    return dict(orgf=lo.astype(f32), invf=f32(inv), invxf=f32(invx), cellf=f32(c), dim=dim, ext=ext, extx=extx,
                r2f=f32(r2))


def coord(g, p, a):
    f = np.floor((f32(p) - g["orgf"][a]) * (g["invxf"] if a == 0 else g["invf"]))
    return int(min(max(f, 0.0), g["dim"][a] - 1))


def row_range(g, q, r2f, yy, zz, lo_x, hi_x):
    c = g["cellf"]
    m = f32(4e-3) * c
    ylo = g["orgf"][1] + f32(yy) * c
    zlo = g["orgf"][2] + f32(zz) * c
    dy = max(f32(0), max(ylo - q[1], q[1] - (ylo + c)) - m)
    dz = max(f32(0), max(zlo - q[2], q[2] - (zlo + c)) - m)
    rem = r2f * f32(1.00002) - dy * dy - dz * dz
    if rem < 0:
        return None
    rx = np.sqrt(rem, dtype=f32) * f32(1.00001)
    fx0 = np.floor((q[0] - rx - g["orgf"][0]) * g["invxf"] - f32(4e-3))
    fx1 = np.floor((q[0] + rx - g["orgf"][0]) * g["invxf"] + f32(4e-3))
    x0 = max(lo_x, int(max(fx0, -1.0)))
    x1 = min(hi_x, int(min(fx1, float(g["dim"][0]))))
    return (x0, x1) if x0 <= x1 else None


def walked_cells(g, queries):
    """Cells (x, y, z) the gather walks for one query or a pair (y and z
    cells at most one apart, x cells at most extx apart; the bounds cover
    both queries' cell ranges)."""
    e = (g["extx"], g["ext"], g["ext"])
    cs = [[coord(g, q[a], a) for a in range(3)] for q in queries]
    lo = [max(min(c[a] for c in cs) - e[a], 0) for a in range(3)]
    hi = [min(max(c[a] for c in cs) + e[a], g["dim"][a] - 1) for a in range(3)]
    cells = set()
    for zz in range(lo[2], hi[2] + 1):
        for yy in range(lo[1], hi[1] + 1):
            rs = [row_range(g, q, g["r2f"], yy, zz, lo[0], hi[0]) for q in queries]
            rs = [r for r in rs if r is not None]
            if not rs:
                continue
            x0, x1 = min(r[0] for r in rs), max(r[1] for r in rs)
            cells.update((x, yy, zz) for x in range(x0, x1 + 1))
    return cells


def shell(rng, q, r2, n):
    """Photons just inside the sphere around q (distance r (1 - 2^-20)),
    where a chord or slab bound that is too tight loses them first."""
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    p = (q.astype(np.float64) + d * np.sqrt(r2) * (1 - 2.0 ** -20)).astype(f32)
    return p[in_radius(q, p, r2)]


def in_radius(q, p, r2):
    d = q.astype(np.float64) - p.astype(np.float64)
    return ((0.0 + d[..., 0] * d[..., 0]) + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2] <= r2


def _boundary_points(rng, g, n):
    """Points on, and a few ulps either side of, cell faces."""
    pts = []
    for _ in range(n):
        p = []
        for a in range(3):
            cw = 1.0 / float(g["invxf"] if a == 0 else g["invf"])
            k = rng.integers(1, g["dim"][a])
            v = f32(float(g["orgf"][a]) + k * cw)
            v = np.nextafter(v, f32(np.inf if rng.random() < 0.5 else -np.inf), dtype=f32) \
                if rng.random() < 0.7 else v
            for _ in range(int(rng.integers(0, 3))):
                v = np.nextafter(v, f32(np.inf), dtype=f32)
            p.append(v)
        pts.append(p)
    return np.array(pts, f32)


@pytest.mark.parametrize("k", [1.0, 2.0])
def test_culled_rows_hold_every_photon_in_radius(k):
    rng = np.random.default_rng(11)
    lo, hi = np.array([-1.0, 0.0, 0.0]), np.array([1.0, 2.0, 2.0])
    r2 = 0.037 ** 2
    g = grid(lo, hi, r2, k=k)
    photons = np.vstack([rng.uniform(lo, hi, (40000, 3)).astype(f32), _boundary_points(rng, g, 4000)])
    queries = np.vstack([rng.uniform(lo + 0.1, hi - 0.1, (150, 3)).astype(f32), _boundary_points(rng, g, 150)])
    pc = [tuple(coord(g, p[a], a) for a in range(3)) for p in photons]
    for q in queries:
        cells = walked_cells(g, [q])
        hit = np.nonzero(in_radius(q, photons, r2))[0]
        missing = [i for i in hit if pc[i] not in cells]
        assert not missing, (q, photons[missing[:3]])
        for p in shell(rng, q, r2, 3000):
            assert tuple(coord(g, p[a], a) for a in range(3)) in cells, (q, p)


@pytest.mark.parametrize("k", [1.0, 2.0])
def test_paired_walk_holds_both_queries_photons(k):
    rng = np.random.default_rng(12)
    lo, hi = np.array([-1.0, 0.0, 0.0]), np.array([1.0, 2.0, 2.0])
    r2 = 0.031 ** 2
    g = grid(lo, hi, r2, k=k)
    photons = np.vstack([rng.uniform(lo, hi, (40000, 3)).astype(f32), _boundary_points(rng, g, 4000)])
    pc = [tuple(coord(g, p[a], a) for a in range(3)) for p in photons]
    pairs = split_x = split_yz = 0
    for _ in range(400):
        a = rng.uniform(lo + 0.1, hi - 0.1).astype(f32)
        b = (a + rng.normal(0, 0.008, 3)).astype(f32)          # a neighbouring pixel's hit point
        if any(abs(coord(g, a[i], i) - coord(g, b[i], i)) > 1 for i in (1, 2)) or \
                abs(coord(g, a[0], 0) - coord(g, b[0], 0)) > g["extx"]:
            continue                                            # the pair walk's condition
        pairs += 1
        split_x += coord(g, a[0], 0) != coord(g, b[0], 0)
        split_yz += any(coord(g, a[i], i) != coord(g, b[i], i) for i in (1, 2))
        cells = walked_cells(g, [a, b])
        for q in (a, b):
            hit = np.nonzero(in_radius(q, photons, r2))[0]
            assert all(pc[i] in cells for i in hit), q
            for p in shell(rng, q, r2, 1000):
                assert tuple(coord(g, p[i], i) for i in range(3)) in cells, (q, p)
    assert pairs > 50 and split_x > 10 and split_yz > 10


def test_sphere_extremes_just_past_a_cell_face_are_walked():
    """Queries placed so that the sphere's extreme point along an axis lies
    a few ulps past a cell face, with a photon just inside the radius there:
    the chord (x) or the row slab (y, z) must still reach that cell."""
    rng = np.random.default_rng(13)
    lo, hi = np.array([-1.0, 0.0, 0.0]), np.array([1.0, 2.0, 2.0])
    for r in (0.0123, 0.037, 0.051):
        r2 = r * r
        g = grid(lo, hi, r2)
        checked = 0
        for _ in range(300):
            a = int(rng.integers(0, 3))
            sgn = 1.0 if rng.random() < 0.5 else -1.0
            cw = 1.0 / float(g["invxf"] if a == 0 else g["invf"])
            k = int(rng.integers(3, g["dim"][a] - 3))
            face = float(g["orgf"][a]) + k * cw
            q = rng.uniform(lo + 0.2, hi - 0.2)
            # the extreme point sits delta past the face, on the far side from q
            delta = float(rng.integers(1, 64)) * 2.0 ** -23 * max(1.0, abs(face))
            q[a] = face - sgn * r + sgn * delta
            q = q.astype(f32)
            p = q.astype(np.float64).copy()
            p[a] += sgn * r * (1 - 2.0 ** -18)
            p = p.astype(f32)
            if not in_radius(q, p[None, :], r2)[0]:
                continue
            cell = tuple(coord(g, p[i], i) for i in range(3))
            assert cell in walked_cells(g, [q]), (r, a, sgn, q, p)
            checked += 1
        assert checked > 150


# ---- the tile gather (k_gather_tile): one walk for a group of hit points,
# rows around the group's box (cell ranges widened by ext from the box's
# corner cells) culled by the box's distance to each row's slab
def box_row_range(g, lo, hi, r2f, yy, zz, lo_x, hi_x):
    c = g["cellf"]
    m = f32(4e-3) * c
    ylo = g["orgf"][1] + f32(yy) * c
    zlo = g["orgf"][2] + f32(zz) * c
    dy = max(f32(0), max(ylo - hi[1], lo[1] - (ylo + c)) - m)
    dz = max(f32(0), max(zlo - hi[2], lo[2] - (zlo + c)) - m)
    rem = r2f * f32(1.00002) - dy * dy - dz * dz
    if rem < 0:
        return None
    rx = np.sqrt(rem, dtype=f32) * f32(1.00001)
    fx0 = np.floor((lo[0] - rx - g["orgf"][0]) * g["invxf"] - f32(4e-3))
    fx1 = np.floor((hi[0] + rx - g["orgf"][0]) * g["invxf"] + f32(4e-3))
    x0 = max(lo_x, int(max(fx0, -1.0)))
    x1 = min(hi_x, int(min(fx1, float(g["dim"][0]))))
    return (x0, x1) if x0 <= x1 else None


def tile_walked_cells(g, group):
    lo = group.min(axis=0).astype(f32)
    hi = group.max(axis=0).astype(f32)
    e = (g["extx"], g["ext"], g["ext"])
    c0 = [max(coord(g, lo[a], a) - e[a], 0) for a in range(3)]
    c1 = [min(coord(g, hi[a], a) + e[a], g["dim"][a] - 1) for a in range(3)]
    cells = set()
    for zz in range(c0[2], c1[2] + 1):
        for yy in range(c0[1], c1[1] + 1):
            rr = box_row_range(g, lo, hi, g["r2f"], yy, zz, c0[0], c1[0])
            if rr is not None:
                cells.update((x, yy, zz) for x in range(rr[0], rr[1] + 1))
    return cells


def _tile_group(rng, lo, hi, r):
    """Hit points of a 4 x 8 pixel tile on a plane through the box (a few
    millimetres apart), sometimes with members up to 2r from the first, as
    the tile gather's grouping allows."""
    centre = rng.uniform(lo + 0.15, hi - 0.15)
    u = rng.normal(size=3)
    u /= np.linalg.norm(u)
    v = np.cross(u, rng.normal(size=3))
    v /= np.linalg.norm(v)
    step = rng.uniform(0.001, 0.006)
    pts = [centre + (i % 4) * step * u + (i // 4) * step * v for i in range(32)]
    if rng.random() < 0.3:
        pts[-1] = centre + rng.uniform(-2 * r, 2 * r, 3)
    return np.array(pts).astype(f32)


@pytest.mark.parametrize("k", [1.0, 2.0])
def test_tile_walk_holds_every_members_photons(k):
    rng = np.random.default_rng(15)
    lo, hi = np.array([-1.0, 0.0, 0.0]), np.array([1.0, 2.0, 2.0])
    r = 0.031
    r2 = r * r
    g = grid(lo, hi, r2, k=k)
    photons = np.vstack([rng.uniform(lo, hi, (40000, 3)).astype(f32), _boundary_points(rng, g, 4000)])
    pc = [tuple(coord(g, p[a], a) for a in range(3)) for p in photons]
    for _ in range(60):
        group = _tile_group(rng, lo, hi, r)
        cells = tile_walked_cells(g, group)
        for q in group:
            hit = np.nonzero(in_radius(q, photons, r2))[0]
            assert all(pc[i] in cells for i in hit), q
            for p in shell(rng, q, r2, 300):
                assert tuple(coord(g, p[a], a) for a in range(3)) in cells, (q, p)


def test_tile_walk_holds_sphere_extremes_just_past_a_cell_face():
    """A member whose sphere's extreme point lies a few ulps past a cell
    face, with a photon just inside the radius there, in a group whose box
    extends away from it: the box's rows and chords must still reach it."""
    rng = np.random.default_rng(16)
    lo, hi = np.array([-1.0, 0.0, 0.0]), np.array([1.0, 2.0, 2.0])
    for r in (0.0123, 0.037):
        r2 = r * r
        g = grid(lo, hi, r2)
        checked = 0
        for _ in range(200):
            a = int(rng.integers(0, 3))
            sgn = 1.0 if rng.random() < 0.5 else -1.0
            cw = 1.0 / float(g["invxf"] if a == 0 else g["invf"])
            kk = int(rng.integers(3, g["dim"][a] - 3))
            face = float(g["orgf"][a]) + kk * cw
            q = rng.uniform(lo + 0.2, hi - 0.2)
            q[a] = face - sgn * r + sgn * float(rng.integers(1, 64)) * 2.0 ** -23 * max(1.0, abs(face))
            q = q.astype(f32)
            p = q.astype(np.float64).copy()
            p[a] += sgn * r * (1 - 2.0 ** -18)
            p = p.astype(f32)
            if not in_radius(q, p[None, :], r2)[0]:
                continue
            others = (q.astype(np.float64) - sgn * np.abs(rng.normal(0, r / 2, (7, 3)))).astype(f32)
            cell = tuple(coord(g, p[i], i) for i in range(3))
            assert cell in tile_walked_cells(g, np.vstack([q[None, :], others])), (r, a, sgn, q, p)
            checked += 1
        assert checked > 100


# ---- the FP64 (plain) path: the same grid in doubles, RowCull<double> and
# CellMath<double>; its kernels are built without FMA contraction, so these
# float64 expressions round as the device's do
def grid64(lo, hi, r2, k=1.0, sx=4):
    g = grid(lo, hi, r2, k, sx)
    r = np.sqrt(r2)
    c = r * ((1.0 + 1.0 / 128.0) / k)
    inv = 1.0 / c
    while int(np.floor((hi[0] - lo[0]) * inv * sx)) + 1 != g["dim"][0]:   # follow the same growth
        c *= 1.25
        inv = 1.0 / c
    return dict(org=lo.astype(np.float64), inv=inv, invx=inv * sx, cell=c, dim=g["dim"], ext=g["ext"],
                extx=g["extx"])


def coord64(g, p, a):
    f = np.floor((p - g["org"][a]) * (g["invx"] if a == 0 else g["inv"]))
    return int(min(max(f, 0.0), g["dim"][a] - 1))


def row_range64(g, q, r2, yy, zz, lo_x, hi_x):
    c = g["cell"]
    m = 1e-6 * c
    ylo = g["org"][1] + yy * c
    zlo = g["org"][2] + zz * c
    dy = max(0.0, max(ylo - q[1], q[1] - (ylo + c)) - m)
    dz = max(0.0, max(zlo - q[2], q[2] - (zlo + c)) - m)
    rem = r2 * (1.0 + 1e-12) - dy * dy - dz * dz
    if rem < 0.0:
        return None
    rx = np.sqrt(rem) * (1.0 + 1e-12)
    fx0 = np.floor((q[0] - rx - g["org"][0]) * g["invx"] - 1e-6)
    fx1 = np.floor((q[0] + rx - g["org"][0]) * g["invx"] + 1e-6)
    x0 = max(lo_x, int(max(fx0, -1.0)))
    x1 = min(hi_x, int(min(fx1, float(g["dim"][0]))))
    return (x0, x1) if x0 <= x1 else None


def walked_cells64(g, q, r2):
    c = [coord64(g, q[a], a) for a in range(3)]
    e = (g["extx"], g["ext"], g["ext"])
    lo = [max(c[a] - e[a], 0) for a in range(3)]
    hi = [min(c[a] + e[a], g["dim"][a] - 1) for a in range(3)]
    cells = set()
    for zz in range(lo[2], hi[2] + 1):
        for yy in range(lo[1], hi[1] + 1):
            rr = row_range64(g, q, r2, yy, zz, lo[0], hi[0])
            if rr is not None:
                cells.update((x, yy, zz) for x in range(rr[0], rr[1] + 1))
    return cells


def test_fp64_culling_holds_sphere_extremes_just_past_a_cell_face():
    rng = np.random.default_rng(14)
    lo, hi = np.array([-1.0, 0.0, 0.0]), np.array([1.0, 2.0, 2.0])
    for r in (0.0123, 0.037, 0.051):
        r2 = r * r
        g = grid64(lo, hi, r2)
        checked = 0
        for _ in range(300):
            a = int(rng.integers(0, 3))
            sgn = 1.0 if rng.random() < 0.5 else -1.0
            cw = 1.0 / (g["invx"] if a == 0 else g["inv"])
            k = int(rng.integers(3, g["dim"][a] - 3))
            face = g["org"][a] + k * cw
            q = rng.uniform(lo + 0.2, hi - 0.2)
            q[a] = face - sgn * r + sgn * float(rng.integers(1, 64)) * 2.0 ** -52 * max(1.0, abs(face))
            p = q.copy()
            p[a] += sgn * r * (1 - 2.0 ** -40)
            if not in_radius(q, p[None, :], r2)[0]:
                continue
            cell = tuple(coord64(g, p[i], i) for i in range(3))
            assert cell in walked_cells64(g, q, r2), (r, a, sgn, q, p)
            checked += 1
        assert checked > 150

"""GPU parity tests: the CUDA path through the C ABI against the FP64 oracle.

Bars (from the hot-path specification):
  - first-hit distances / object ids for fixed ray sets: FP64 bit-exact;
    FP32 ids exact away from ties, t within 1e-5 relative;
  - photons traced on the GPU (FP64) equal the oracle's for the same stream;
  - in-radius neighbour sets equal the f64 kd-tree predicate bit for bit
    (FP64 map and FP32 map);
  - per-hit-point radiance sums within 1e-5 relative (FP64: 1e-9);
  - one FP64 pass image equals the oracle's recursive trace_ray evaluation
    within 1e-9 relative.
"""
import numpy as np
import pytest

from oracle.binding import Oracle
from ppmpa_gb300 import MIXED, PLAIN, Context, PPMError, RenderConfig, scene as S, workloads as W

pytestmark = pytest.mark.gpu

SCENES = {
    "box_c1": (lambda: S.box_scene("c1"), lambda: S.box_camera(48)),
    "box_c2": (lambda: S.box_scene("c2"), lambda: S.box_camera(48)),
    "reference": (S.reference_scene, lambda: S.make_camera(40, 40)),
}


@pytest.fixture(scope="module")
def ctx():
    c = Context(0, seed=1234)
    yield c
    c.close()


def _setup(ctx, name):
    sc, cam = SCENES[name][0](), SCENES[name][1]()
    ctx.upload_scene(sc)
    ctx.set_camera(cam)
    return sc, cam, Oracle(sc, cam)


def _random_rays(rng, n, lo, hi):
    p = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.hstack([p, d])


@pytest.mark.parametrize("name", list(SCENES))
def test_intersect_fp64_bit_exact(ctx, name):
    sc, cam, orc = _setup(ctx, name)
    rng = np.random.default_rng(1)
    lo, hi = ((-0.99, 0.01, 0.01), (0.99, 1.99, 1.99)) if name != "reference" else ((-1.9, 0.1, -4.9), (1.9, 3.9, 5.9))
    rays = _random_rays(rng, 20000, lo, hi)
    t, obj, nrm = ctx.intersect(rays)
    ot, oobj, onrm, _ = orc.intersect(rays)
    assert np.array_equal(obj, oobj)
    assert np.array_equal(t, ot)
    assert np.array_equal(nrm, onrm)
    assert (obj >= 0).mean() > 0.5


@pytest.mark.parametrize("name", list(SCENES))
def test_intersect_fp32_ids_and_distances(ctx, name):
    sc, cam, orc = _setup(ctx, name)
    rng = np.random.default_rng(2)
    lo, hi = ((-0.99, 0.01, 0.01), (0.99, 1.99, 1.99)) if name != "reference" else ((-1.9, 0.1, -4.9), (1.9, 3.9, 5.9))
    rays = _random_rays(rng, 20000, lo, hi)
    t, obj = ctx.intersect(rays, f32=True)
    ot, oobj, onrm, _ = orc.intersect(rays)
    same = obj == oobj
    assert same.mean() > 0.999
    hit = same & (obj >= 0)
    # FP32 conditioning: t = -(d + n.o)/(n.dir) carries an absolute error of a few
    # ulps of the scene scale divided by |cos| at the hit (grazing rays)
    cos = np.abs(np.einsum("ij,ij->i", onrm, rays[:, 3:]))
    scale = np.abs(rays[:, :3]).max(1) + np.abs(ot) + 6.0
    tol = 1e-5 * np.abs(ot) + 8 * 2.0 ** -24 * scale / np.maximum(cos, 1e-6)
    assert (np.abs(t - ot)[hit] <= tol[hit]).all()
    assert np.allclose(t[hit & (cos > 0.05)], ot[hit & (cos > 0.05)], rtol=1e-5, atol=1e-5)
    # id mismatches only where the FP64 ray hits a different object at a
    # nearly equal distance (an FP32 tie) -- check the FP32 choice is that close
    for i in np.nonzero(~same)[0]:
        if obj[i] >= 0 and oobj[i] >= 0:
            assert abs(t[i] - ot[i]) <= 1e-3 * max(1.0, ot[i])


@pytest.mark.parametrize("name,uc", [("box_c1", True), ("box_c1", False), ("box_c2", True), ("reference", True)])
def test_trace_photons_fp64_match_oracle(ctx, name, uc):
    sc, cam, orc = _setup(ctx, name)
    for pass_index in (0, 3):
        g = ctx.trace_photons(20000, use_classic=uc, pass_index=pass_index)
        o = orc.trace_photons(20000, use_classic=uc, seed=1234, pass_index=pass_index)
        assert g["power"] == o["power"] and g["n_emitted"] == o["n_emitted"]
        kg = np.lexsort((g["level"], g["emit"]))
        ko = np.lexsort((o["level"], o["emit"]))
        assert len(kg) == len(ko)
        assert np.array_equal(g["emit"][kg], o["emit"][ko])
        assert np.array_equal(g["level"][kg], o["level"][ko])
        assert np.array_equal(g["wl"][kg], o["wl"][ko])
        assert np.array_equal(g["pos"][kg], o["pos"][ko])
        assert np.array_equal(g["dir"][kg], o["dir"][ko])


def _photon_cloud(rng, n, clustered=False):
    pos = rng.random((n, 3))
    if clustered:
        centres = rng.random((50, 3))
        k = int(0.9 * n)
        pos[:k] = centres[rng.integers(0, 50, k)] + rng.normal(0, 0.01, (k, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    wl = rng.integers(0, 3, n).astype(np.uint8)
    return pos, d, wl


@pytest.mark.parametrize("clustered", [False, True])
def test_within_fp64_sets_equal(ctx, clustered):
    rng = np.random.default_rng(5)
    pos, d, wl = _photon_cloud(rng, 60000, clustered)
    R2 = 0.03 ** 2
    ctx.build_photonmap(pos, d, wl, 0.01, R2)
    q = np.vstack([rng.random((3000, 3)), pos[rng.integers(0, len(pos), 1000)]])
    r2 = np.concatenate([np.full(2000, R2), rng.uniform(0, R2, len(q) - 2000)])
    off, idx = ctx.query_within(q, r2)
    ooff, oidx = Oracle(S.Scene()).within(pos, q, r2)
    assert np.array_equal(off, ooff)
    assert np.array_equal(idx, oidx)
    assert len(idx) > 10000


def test_within_fp64_boundary_equality(ctx):
    # photons placed exactly at distance^2 == r2 (in f64) are inside (<=)
    pos = np.array([[0.5, 0.5, 0.5], [0.75, 0.5, 0.5], [0.5, 0.25, 0.5], [0.5, 0.5, 0.8]])
    d = np.tile([0.0, 0.0, -1.0], (4, 1))
    wl = np.zeros(4, np.uint8)
    ctx.build_photonmap(pos, d, wl, 1.0, 0.0625)
    off, idx = ctx.query_within(np.array([[0.5, 0.5, 0.5]]), 0.0625)
    assert sorted(idx.tolist()) == [0, 1, 2]


def test_estimate_fp64(ctx):
    rng = np.random.default_rng(6)
    pos, d, wl = _photon_cloud(rng, 50000)
    R2 = 0.04 ** 2
    ctx.build_photonmap(pos, d, wl, 0.002, R2)
    q = rng.random((4000, 3))
    n = rng.normal(size=(4000, 3))
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    orc = Oracle(S.Scene())
    for pf in (S.FILTER_NONE, S.FILTER_CONE, S.FILTER_GAUSS):
        g = ctx.estimate(q, n, pf)
        o = orc.estimate(pos, d, wl, q, n, R2, 0.002, pf)
        assert np.allclose(g, o, rtol=1e-9, atol=1e-12), pf
        assert (o > 0).mean() > 0.3


_oct_roundtrip = W.oct_roundtrip


@pytest.mark.parametrize("clustered", [False, True])
def test_fp32_map_sets_and_estimates(ctx, clustered):
    rng = np.random.default_rng(7)
    pos, d, wl = _photon_cloud(rng, 80000, clustered)
    pos32 = pos.astype(np.float32)
    R2max = 0.03 ** 2
    ctx.build_photonmap_f32(pos32, d.astype(np.float32), wl, 0.003, R2max)
    q32 = np.vstack([rng.random((3000, 3)), pos[rng.integers(0, len(pos), 1000)]]).astype(np.float32)
    r2 = np.exp(rng.uniform(np.log(1e-6), np.log(R2max), len(q32)))
    off, idx = ctx.query_within_f32(q32, r2)
    orc = Oracle(S.Scene())
    ooff, oidx = orc.within(pos32.astype(np.float64), q32.astype(np.float64), r2)
    assert np.array_equal(off, ooff)
    assert np.array_equal(idx, oidx)
    n = rng.normal(size=(len(q32), 3))
    n = (n / np.linalg.norm(n, axis=1, keepdims=True)).astype(np.float32)
    g = ctx.estimate_f32(q32, n, r2)
    dq = _oct_roundtrip(d)
    for i in range(0, len(q32), 397):
        o = orc.estimate(pos32.astype(np.float64), dq, wl, q32[i:i + 1].astype(np.float64),
                         n[i:i + 1].astype(np.float64), r2[i], 0.003)
        assert np.allclose(g[i], o[0], rtol=1e-5, atol=1e-9), i


@pytest.mark.parametrize("name,uc", [("box_c1", True), ("box_c2", True), ("box_c1", False), ("reference", True)])
def test_fp64_pass_image_matches_oracle(ctx, name, uc):
    sc, cam, orc = _setup(ctx, name)
    r0 = 0.08 if name != "reference" else 0.2
    cfg = RenderConfig(nphoton=20000, passes=1, use_classic=uc, radius0=r0, alpha=0.7, precision=PLAIN,
                       use_graph=False, seed=1234)
    ctx.render_begin(cfg)
    ctx.render_step(1)
    img = ctx.render_pass_image()
    ph = orc.trace_photons(20000, use_classic=uc, seed=1234, pass_index=0)
    oimg = orc.eye_pass(ph, r0 * r0, use_classic=uc, seed=1234, pass_index=0)
    assert np.allclose(img, oimg, rtol=1e-9, atol=1e-12 * max(1.0, oimg.max()))
    assert oimg.max() > 0


def test_render_graph_equals_eager(ctx):
    sc, cam, orc = _setup(ctx, "box_c2")
    imgs = []
    for g in (False, True):
        for prec in (PLAIN, MIXED):
            cfg = RenderConfig(nphoton=20000, passes=3, radius0=0.08, precision=prec, use_graph=g, seed=99)
            imgs.append(ctx.render(cfg))
    assert np.allclose(imgs[0], imgs[2], rtol=1e-9, atol=1e-14)
    assert np.allclose(imgs[1], imgs[3], rtol=1e-5, atol=1e-12)


def test_ray_counters(ctx):
    """photon_rays counts one segment per photon event, eye_rays the eye-tree
    rays; both are per pass and reproducible for a fixed seed."""
    sc, cam, orc = _setup(ctx, "box_c1")
    npx = cam.xreso * cam.yreso
    seen = []
    for g in (False, True):
        cfg = RenderConfig(nphoton=20000, passes=2, radius0=0.08, precision=PLAIN, use_graph=g, seed=11)
        ctx.render(cfg)
        st = ctx.stats()
        assert st["photons_emitted"] <= st["photon_rays"] <= 10 * st["photons_emitted"]
        assert st["photons_stored"] <= st["photon_rays"]
        assert npx < st["eye_rays"] < 10 * npx          # the mirror sphere spawns children
        seen.append((st["photon_rays"], st["eye_rays"]))
    assert seen[0] == seen[1]


def test_mixed_matches_plain_statistically(ctx):
    sc, cam, orc = _setup(ctx, "box_c1")
    plain = ctx.render(RenderConfig(nphoton=50000, passes=8, radius0=0.08, precision=PLAIN, seed=5))
    mixed = ctx.render(RenderConfig(nphoton=50000, passes=8, radius0=0.08, precision=MIXED, seed=5))
    ref = ctx.render(RenderConfig(nphoton=50000, passes=64, radius0=0.08, precision=PLAIN, seed=77))
    e_plain = np.sqrt(np.mean((plain - ref) ** 2))
    e_mixed = np.sqrt(np.mean((mixed - ref) ** 2))
    assert abs(plain.mean() / ref.mean() - 1) < 0.05
    assert abs(mixed.mean() / ref.mean() - 1) < 0.05
    assert e_mixed < 1.1 * e_plain


def test_error_paths(ctx):
    with pytest.raises(PPMError) as e:
        ctx.build_photonmap(np.zeros((1, 3)), np.zeros((1, 3)), np.array([5], np.uint8), 1.0, 0.01)
    assert e.value.status == 1
    ctx.build_photonmap(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0, np.uint8), 1.0, 0.01)
    off, idx = ctx.query_within(np.zeros((2, 3)), 0.01)
    assert off.tolist() == [0, 0, 0] and len(idx) == 0
    assert np.all(ctx.estimate(np.zeros((2, 3)), np.tile([0, 1, 0], (2, 1))) == 0)
    with pytest.raises(PPMError) as e:
        ctx.query_within(np.zeros((1, 3)), 0.02)        # beyond the map radius
    assert e.value.status == 1
    bad = S.Scene()
    m = bad.add_material(S.new_simple((1, 1, 1), (0, 0, 0), 1, 0, 0))
    bad.add(S.sphere((0, 0, 0), 1), m + 5)
    with pytest.raises(PPMError) as e:
        ctx.upload_scene(bad)
    assert e.value.status == 1



def test_cell_factors_give_the_same_image(ctx):
    # the grid granularity changes which candidates are tested, never the
    # in-radius sets; images agree up to FP32 summation order
    sc, cam, orc = _setup(ctx, "box_c2")
    imgs = []
    for prec in (MIXED, PLAIN):
        for cf in (1, 2):
            cfg = RenderConfig(nphoton=30000, passes=1, radius0=0.08, precision=prec, use_graph=False, seed=21,
                               cell_factor=cf)
            ctx.render_begin(cfg)
            ctx.render_step(1)
            imgs.append(ctx.render_pass_image())
    assert np.allclose(imgs[1], imgs[0], rtol=2e-5, atol=1e-7 * imgs[0].max())
    assert np.allclose(imgs[3], imgs[2], rtol=1e-12, atol=1e-14 * imgs[2].max())
    assert imgs[0].max() > 0


def test_cli_renders_one_pass_in_reference_format(built_lib):
    import subprocess
    from ppmpa_gb300 import build as lib_build
    out = subprocess.run([lib_build.CLI, "20000", "0.2", "cam.scr", "scene.scene"], capture_output=True, text=True,
                         check=True, timeout=120)
    lines = out.stdout.split("\n")
    assert lines[0] == "P3" and lines[1] == "## max radiance = 0.01"
    assert lines[2] == "## image parameters = 1/250, F4, ISO100" and lines[3] == "256 256" and lines[4] == "255"
    px = [l.split() for l in lines[5:5 + 256 * 256]]
    assert len(px) == 65536 and all(len(p) == 3 for p in px)
    vals = np.array([[float(v) for v in p] for p in px])
    assert np.isfinite(vals).all() and vals.max() > 0


def test_c1_full_configuration_render_matches_oracle(ctx):
    """The diffuse-sphere box at its full configuration (256x256, 200k
    photons per pass, r0 0.05, alpha 0.7, 10 passes), plain FP64 with the
    pass graph: the averaged image equals the oracle's progressive render
    (photon traces, radius schedule, eye passes, average) within 1e-9."""
    sc, cam = S.box_scene("c1"), S.box_camera(256)
    ctx.upload_scene(sc)
    ctx.set_camera(cam)
    cfg = RenderConfig(nphoton=200_000, passes=10, radius0=0.05, alpha=0.7, precision=PLAIN, seed=1234)
    got = ctx.render(cfg)
    want = Oracle(sc, cam).render(200_000, 10, 0.05, 0.7, schedule_offset=1, use_classic=True, seed=1234)
    assert want.max() > 0
    assert np.allclose(got, want, rtol=1e-9, atol=1e-12 * want.max())
    mixed = ctx.render(RenderConfig(nphoton=200_000, passes=10, radius0=0.05, alpha=0.7, precision=MIXED, seed=1234))
    assert abs(mixed.mean() / want.mean() - 1) < 0.02


def test_not_ready_and_capacity_errors():
    """Render calls out of order report NOT_READY; a caller index buffer too
    small reports CAPACITY; an eye tree wider than its per-level queues
    is reported as CAPACITY instead of a silently truncated image: both
    children of every front hit on the inner ball reach glass again, four
    vertices per pixel at the second level against room for two."""
    import ctypes as C
    from ppmpa_gb300 import _lib
    with Context(0, seed=3) as fresh:
        with pytest.raises(PPMError) as e:
            fresh.render(RenderConfig(nphoton=1000, passes=1))
        assert e.value.status == 6
        with pytest.raises(PPMError) as e:
            fresh.render_step(1)
        assert e.value.status == 6
        rng = np.random.default_rng(8)
        pos, d, wl = _photon_cloud(rng, 2000)
        fresh.build_photonmap(pos, d, wl, 1.0, 0.2 ** 2)
        q = np.array([[0.5, 0.5, 0.5]])
        r2 = np.array([0.2 ** 2])
        off = np.zeros(2, np.int64)
        idx = np.zeros(1, np.int32)
        tot = C.c_int64()
        lib = _lib.load()
        st = lib.ppm_query_within(fresh.h, q.ctypes.data_as(C.POINTER(C.c_double)), 1,
                                  r2.ctypes.data_as(C.POINTER(C.c_double)), off.ctypes.data_as(C.POINTER(C.c_int64)),
                                  idx.ctypes.data_as(C.POINTER(C.c_int32)), 1, C.byref(tot))
        assert st == 3 and tot.value > 1

        sc = S.Scene()
        white = sc.add_material(S.new_simple((0.75, 0.75, 0.75), (0.0, 0.0, 0.0), 1.0, 0.0, 0.0))
        glass = sc.add_material(S.new_ts((1.0, 1.0, 1.0), (0.05, 0.05, 0.05), 0.0, 0.0, 0.0, ior=(1.5, 1.5, 1.5)))
        sc.add(S.sphere((0.0, 1.0, 1.0), 5.0), glass)          # the camera sits inside this glass shell
        sc.add(S.sphere((0.0, 1.0, 1.0), 2.0), glass)          # and looks at a second glass ball filling the view
        sc.add(S.parallelogram((-9.0, -9.0, 9.0), (9.0, -9.0, 9.0), (-9.0, 9.0, 9.0)), white)
        sc.lights.append(S.point_light(S.color_normalize((1, 1, 1)), 100.0, (0.0, 1.0, 3.0)))
        fresh.upload_scene(sc)
        fresh.set_camera(S.box_camera(32))
        with pytest.raises(PPMError) as e:
            fresh.render(RenderConfig(nphoton=2000, passes=1, radius0=0.1, precision=PLAIN, seed=3))
        assert e.value.status == 3 and "overflow" in str(e.value)

"""The GPU-built BVH and the large-mesh scene (a displaced icosphere of up to
1.31M triangles in the box, lit by a spot light).

Bars:
  - with the hierarchy, first hits equal the reference's loop over all
    objects: FP64 ids, distances and normals bit for bit against the oracle,
    and on the GPU the hierarchy and the loop agree bit for bit in both
    precisions (nearest t, ties to the lower index);
  - photons traced through a mesh scene lit by the spot light equal the
    oracle's photon for photon (FP64);
  - the full 1.31M-triangle scene builds and renders.
"""
import numpy as np
import pytest

from oracle.binding import Oracle
from ppmpa_gb300 import MIXED, PLAIN, Context, RenderConfig, mesh as M, scene as S

pytestmark = pytest.mark.gpu
BVH, LOOP = 1, 2


@pytest.fixture(scope="module")
def ctx():
    c = Context(0, seed=4321)
    yield c
    c.close()


def _rays(rng, n):
    p = rng.uniform((-0.95, 0.05, 0.05), (0.95, 1.95, 1.95), (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.hstack([p, d])


@pytest.mark.parametrize("level,nrays,leaf", [(1, 20000, 1), (4, 20000, 1), (6, 4000, 1), (4, 20000, 2),
                                              (4, 20000, 4), (6, 4000, 8), (1, 2000, 8)])
def test_bvh_first_hits_match_oracle_loop(ctx, level, nrays, leaf):
    sc = M.mesh_scene(level)
    ctx.set_bvh_leaf(leaf)
    ctx.upload_scene(sc)
    ctx.set_accel(BVH)
    assert ctx.accel_info()["bvh_objects"] == sc.n_objects
    rays = _rays(np.random.default_rng(level), nrays)
    t, obj, nrm = ctx.intersect(rays)
    ot, oobj, onrm, _ = Oracle(sc).intersect(rays)
    assert np.array_equal(obj, oobj)
    assert np.array_equal(t, ot)
    assert np.array_equal(nrm, onrm)
    assert (obj >= 5).mean() > 0.05         # rays do reach the mesh


@pytest.mark.parametrize("scene", ["box_c2", "mesh5"])
def test_bvh_equals_loop_on_gpu_both_precisions(ctx, scene):
    sc = S.box_scene("c2") if scene == "box_c2" else M.mesh_scene(5)
    ctx.upload_scene(sc)
    rays = _rays(np.random.default_rng(11), 50000)
    out = {}
    for mode in (BVH, LOOP):
        ctx.set_accel(mode)
        out[mode] = (ctx.intersect(rays), ctx.intersect(rays, f32=True))
    (t1, o1, n1), (tf1, of1) = out[BVH]
    (t2, o2, n2), (tf2, of2) = out[LOOP]
    assert np.array_equal(o1, o2) and np.array_equal(t1, t2) and np.array_equal(n1, n2)
    assert np.array_equal(of1, of2) and np.array_equal(tf1, tf2)


def test_spot_light_photons_through_bvh_match_oracle(ctx):
    sc = M.mesh_scene(3)
    cam = S.box_camera(32)
    ctx.upload_scene(sc)
    ctx.set_camera(cam)
    ctx.set_accel(BVH)
    orc = Oracle(sc, cam)
    for pass_index in (0, 2):
        g = ctx.trace_photons(5000, use_classic=True, pass_index=pass_index)
        o = orc.trace_photons(5000, use_classic=True, seed=4321, pass_index=pass_index)
        assert g["power"] == o["power"] and g["n_emitted"] == o["n_emitted"]
        kg = np.lexsort((g["level"], g["emit"]))
        ko = np.lexsort((o["level"], o["emit"]))
        assert len(kg) == len(ko) > 1000
        for k in ("emit", "level", "wl", "pos", "dir"):
            assert np.array_equal(g[k][kg], o[k][ko]), k


def test_full_mesh_builds_and_renders(ctx):
    sc = M.mesh_scene(8)
    ctx.upload_scene(sc)
    ctx.set_accel(0)
    assert ctx.accel_info()["bvh_objects"] == 1_310_725
    rays = _rays(np.random.default_rng(3), 400)
    t, obj, nrm = ctx.intersect(rays)
    ot, oobj, onrm, _ = Oracle(sc).intersect(rays)
    assert np.array_equal(obj, oobj) and np.array_equal(t, ot)
    ctx.set_camera(S.box_camera(256))
    imgs = [ctx.render(RenderConfig(nphoton=200_000, passes=2, radius0=0.05, alpha=0.7, precision=p, seed=9))
            for p in (PLAIN, MIXED)]
    for img in imgs:
        assert np.isfinite(img).all() and img.mean() > 0
    assert abs(imgs[1].mean() / imgs[0].mean() - 1) < 0.1


def test_leaf_tuner_keeps_answers(ctx):
    sc = M.mesh_scene(5)
    ctx.set_bvh_leaf(1)
    ctx.upload_scene(sc)
    ctx.set_accel(0)
    rays = _rays(np.random.default_rng(21), 30000)
    want = ctx.intersect(rays)
    leaf, ms = ctx.tune_bvh_leaf(rays)
    assert leaf in (1, 2, 4, 8) and ms > 0
    got = ctx.intersect(rays)
    assert all(np.array_equal(a, b) for a, b in zip(got, want))
    ctx.set_bvh_leaf(1)


@pytest.mark.parametrize("n_prims,leaf", [(3000, 1), (3000, 4), (200, 2)])
def test_bvh_on_spheres_and_quads_matches_oracle(ctx, n_prims, leaf):
    """Batch-workload scenes: spheres and parallelograms in random positions
    and orientations (sphere roots, parallelogram bounds, ties between
    overlapping objects) through the hierarchy, against the oracle's loop."""
    from ppmpa_gb300 import workloads as W
    sc = W.batch_scene(np.random.default_rng(n_prims + leaf), n_prims)
    ctx.set_bvh_leaf(leaf)
    ctx.upload_scene(sc)
    ctx.set_accel(BVH)
    rays = _rays(np.random.default_rng(77), 20000)
    t, obj, nrm = ctx.intersect(rays)
    ot, oobj, onrm, _ = Oracle(sc).intersect(rays)
    assert np.array_equal(obj, oobj) and np.array_equal(t, ot) and np.array_equal(nrm, onrm)
    assert (obj >= 5).mean() > 0.05
    ctx.set_bvh_leaf(1)


def test_render_through_the_loop_and_the_hierarchy_agree(ctx):
    """A scene of 45 objects rendered with the loop over its objects (a table
    too large for the eye levels' shared-memory copy, so they read it from
    global memory) and through the hierarchy: the same first hits, so the
    same image up to the order of FP32 sums."""
    from ppmpa_gb300 import workloads as W
    sc = W.batch_scene(np.random.default_rng(40), 40)
    assert sc.n_objects > 32
    ctx.upload_scene(sc)
    ctx.set_camera(S.box_camera(128))
    imgs = []
    for mode in (LOOP, BVH):
        ctx.set_accel(mode)
        imgs.append(ctx.render(RenderConfig(nphoton=100_000, passes=2, radius0=0.05, alpha=0.7, precision=MIXED,
                                            seed=3)))
    ctx.set_accel(0)
    assert np.isfinite(imgs[0]).all() and imgs[0].mean() > 0
    assert np.allclose(imgs[0], imgs[1], rtol=1e-4, atol=1e-6 * imgs[0].max())

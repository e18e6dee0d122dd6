"""Batched rendering (ppm_batch_render): every job's image equals the image
ppm_render gives for that job alone (same seed and configuration), up to the
order of floating-point atomic adds; jobs with fewer passes drop out at the
right pass; the cell-size autotuner changes nothing but speed."""
import numpy as np
import pytest

from ppmpa_gb300 import MIXED, PLAIN, Batch, Context, RenderConfig, mesh as M, scene as S, workloads as W

pytestmark = pytest.mark.gpu


def _jobs():
    rng = np.random.default_rng(3)
    return [
        (S.box_scene("c1"), S.box_camera(64), RenderConfig(nphoton=30000, passes=4, radius0=0.08, seed=11)),
        (S.box_scene("c2"), S.box_camera(96), RenderConfig(nphoton=50000, passes=2, radius0=0.06, alpha=0.5,
                                                           precision=PLAIN, seed=12)),
        (M.mesh_scene(3), S.box_camera(80), RenderConfig(nphoton=40000, passes=3, radius0=0.07, seed=13)),
        (W.batch_scene(rng, 3000), S.box_camera(72), RenderConfig(nphoton=20000, passes=5, radius0=0.05, seed=14)),
        (W.batch_scene(rng, 40), S.box_camera(64), RenderConfig(nphoton=60000, passes=1, radius0=0.09, seed=15,
                                                               precision=PLAIN)),
    ]


def test_batch_images_equal_single_renders():
    jobs = _jobs()
    with Batch(0, seed=1) as b:
        imgs, ms = b.render(jobs)
    assert ms > 0
    with Context(0, seed=1) as ctx:
        for (sc, cam, cfg), img in zip(jobs, imgs):
            ctx.upload_scene(sc)
            ctx.set_camera(cam)
            want = ctx.render(cfg)
            tol = 1e-10 if cfg.precision == PLAIN else 1e-5
            assert img.shape == want.shape
            assert np.allclose(img, want, rtol=tol, atol=tol * want.max()), cfg
            assert want.max() > 0


def _mixed_jobs():
    """Mixed-precision photon-mapping jobs of every kind a staged batch takes:
    small and large images, a mesh walked through its BVH, a parallelogram
    light, uneven photon budgets and pass counts."""
    rng = np.random.default_rng(5)
    return [
        (S.box_scene("c1"), S.box_camera(64), RenderConfig(nphoton=30000, passes=4, radius0=0.08, seed=21)),
        (S.box_scene("c2"), S.box_camera(96), RenderConfig(nphoton=50000, passes=2, radius0=0.06, alpha=0.5,
                                                           seed=22)),
        (M.mesh_scene(3), S.box_camera(80), RenderConfig(nphoton=40000, passes=3, radius0=0.07, seed=23)),
        (W.batch_scene(rng, 3000), S.box_camera(72), RenderConfig(nphoton=20000, passes=5, radius0=0.05, seed=24)),
        (W.batch_scene(rng, 40), S.box_camera(40), RenderConfig(nphoton=60000, passes=1, radius0=0.09, seed=25,
                                                               flags=1)),
    ]


def test_staged_batch_images_equal_single_renders():
    """One launch per stage over all jobs gives each job the image of its own
    render (the same paths and neighbour sets; FP32 sums in another order)."""
    from ppmpa_gb300.api import BATCH_STAGED
    jobs = _mixed_jobs()
    with Batch(0, seed=1) as b:
        b.set_mode(BATCH_STAGED)
        imgs, ms = b.render(jobs)
        info = b.info()
    assert info["staged"] and info["tile"] > 0 and ms > 0
    with Context(0, seed=1) as ctx:
        for (sc, cam, cfg), img in zip(jobs, imgs):
            ctx.upload_scene(sc)
            ctx.set_camera(cam)
            want = ctx.render(cfg)
            assert img.shape == want.shape
            assert np.allclose(img, want, rtol=1e-5, atol=1e-5 * want.max()), cfg
            assert want.max() > 0


def test_staged_and_graph_batches_agree():
    from ppmpa_gb300.api import BATCH_GRAPHS, BATCH_STAGED
    jobs = _mixed_jobs()[:3]
    out = {}
    with Batch(0, seed=1) as b:
        for mode in (BATCH_STAGED, BATCH_GRAPHS):
            b.set_mode(mode, tile=4096)
            out[mode], _ = b.render(jobs)
            assert b.info()["staged"] == (mode == BATCH_STAGED)
    for a, g in zip(out[BATCH_STAGED], out[BATCH_GRAPHS]):
        assert np.allclose(a, g, rtol=1e-5, atol=1e-5 * g.max())


def test_staged_batch_refuses_plain_jobs():
    from ppmpa_gb300 import PPMError
    from ppmpa_gb300.api import BATCH_STAGED
    with Batch(0, seed=1) as b:
        b.set_mode(BATCH_STAGED)
        with pytest.raises(PPMError, match="staged batch passes"):
            b.render(_jobs()[:2])


def test_cell_tuning_changes_only_speed():
    sc, cam = S.box_scene("c2"), S.box_camera(96)
    with Context(0, seed=1) as ctx:
        ctx.upload_scene(sc)
        ctx.set_camera(cam)
        base = dict(nphoton=50000, passes=3, radius0=0.06, seed=21, precision=MIXED)
        imgs = {cf: ctx.render(RenderConfig(cell_factor=cf, **base)) for cf in (1, 2)}
        tuned = ctx.render(RenderConfig(flags=1, **base))
        cf = ctx.stats()["cell_factor"]
        assert cf in (1, 2)
        assert np.allclose(tuned, imgs[cf], rtol=1e-5, atol=1e-5 * tuned.max())


@pytest.mark.parametrize("precision,tol", [(PLAIN, 1e-12), (MIXED, 1e-6)])
def test_pass_shards_reassemble_the_full_render(precision, tol):
    """Passes rendered in blocks (first_pass) and averaged give the image of
    one render of all passes: the pass-sharded multi-GPU path, run as two
    shards one after another on one GPU."""
    from ppmpa_gb300.shard import context_renderer, render_sharded
    sc, cam = S.box_scene("c2"), S.box_camera(64)
    cfg = RenderConfig(nphoton=30000, passes=6, radius0=0.08, precision=precision, seed=31)
    with Context(0, seed=1) as ctx:
        ctx.upload_scene(sc)
        ctx.set_camera(cam)
        full = ctx.render(cfg)
        run = context_renderer(ctx, cfg)
        parts = [render_sharded(run, 6, r, 2, reduce_sum=lambda a: a) for r in range(2)]
        # rank 0's block plus rank 1's block, as the reduction would add them
        from ppmpa_gb300.shard import shard_passes
        total = sum(run(*shard_passes(6, r, 2)) for r in range(2)) / 6.0
    assert np.allclose(total, full, rtol=tol, atol=tol * full.max())
    assert parts[1] is None


def test_auto_mode_times_both_modes_and_keeps_the_faster():
    """PPM_BATCH_AUTO times one pass of each mode on the first render and
    keeps the faster one; either way every job gets its own image."""
    jobs = _mixed_jobs()[:3]
    with Batch(0, seed=1) as b:
        imgs, _ = b.render(jobs)
        info = b.info()
        t = info["trial_ms"]
        assert t["staged"] > 0 and t["graphs"] > 0
        assert info["staged"] == (t["staged"] <= t["graphs"])
        again, _ = b.render(jobs)
        assert b.info()["staged"] == info["staged"]
    for a, c in zip(imgs, again):
        assert np.allclose(a, c, rtol=1e-5, atol=1e-5 * c.max())

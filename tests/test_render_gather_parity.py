"""The mixed render's own gather, hit point by hit point, against the oracle.

ppm_render_gather_export runs one pass of a mixed-precision render with the
render gather's per-hit-point records on, and returns that pass's sorted
FP32 photon map, its hit points and, per hit point, what the gather found:
the number of photons in radius, a checksum of their slots in the map and
the FP32 flux sums per wavelength.  The oracle (orc_gather_sums) restates
estimate_radiance (src/tracer.rs:179-216) in FP64 on the same FP32 values:
the same photon positions, the directions decoded from the same packed
words, the same hit points, the pass's radius^2.

Bars:
  - in-radius counts and set checksums equal, bit for bit (the neighbour
    set of the kdtree crate's f64 predicate);
  - flux sums within 1e-5 relative, with an absolute floor of 1e-6 per
    photon in radius (one FP32 cosine carries about 3e-7 of error, so a sum
    of near-grazing photons has no meaningful relative bar); and at least
    99.9 % of the non-zero sums within 1e-5 relative alone;
  - the FP32 gathered-flux image equals the sum over each pixel's hit points
    of weight x sums within 1e-5 relative (order of the FP32 atomic adds).

Cases: the glass box (512 x 512, 1M photons per pass) at pass 0 and pass 33
with 1 and 2 cells per radius, the cone and Gauss filters at pass 33, and
the diffuse-sphere box (256 x 256, 200k photons) at its full size; each for
the default row-walk gather and for the tile gather (PPM_RENDER_TILE_GATHER).
"""
import numpy as np
import pytest

from oracle.binding import Oracle
from ppmpa_gb300 import MIXED, Context, RenderConfig, scene as S
from ppmpa_gb300.api import RENDER_TILE_GATHER

GATHERS = {"row_walk": 0, "tile": RENDER_TILE_GATHER}

pytestmark = pytest.mark.gpu

SUM_RTOL = 1e-5
SUM_ATOL_PER_PHOTON = 1e-6


def decode_photons(ph):
    """Positions (float64 of the FP32 values), unit directions decoded from the
    15+15-bit octahedral words as the gather decodes them (FP32 arithmetic,
    then normalised in FP64) and wavelengths."""
    word = ph[:, 3].copy().view(np.uint32)
    c = np.float32(2.0) / np.float32(32767.0)
    px = (word & 32767).astype(np.float32) * c - np.float32(1.0)
    py = ((word >> 15) & 32767).astype(np.float32) * c - np.float32(1.0)
    pz = np.float32(1.0) - np.abs(px) - np.abs(py)
    t = np.maximum(-pz, np.float32(0.0))
    px = px - np.copysign(t, px)
    py = py - np.copysign(t, py)
    d = np.stack([px, py, pz], axis=1).astype(np.float64)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return ph[:, :3].astype(np.float64), d, (word >> 30).astype(np.uint8)


def check_export(ex, orc):
    pos, d, wl = decode_photons(ex["photons"])
    hits = ex["hits"]
    q, n, w = hits[:, 0:3], hits[:, 3:6], hits[:, 6:9]
    pixel = hits[:, 9].copy().view(np.int32)
    count, check, sums = orc.gather_sums(pos, d, wl, q, n, ex["radius2"], ex["pfilter"])
    g_count = ex["counts"].astype(np.int64)
    assert np.array_equal(g_count, count), f"{(g_count != count).sum()} hit points with other in-radius counts"
    assert np.array_equal(ex["checksums"], check), f"{(ex['checksums'] != check).sum()} neighbour sets differ"
    g = ex["sums"].astype(np.float64)
    err = np.abs(g - sums)
    tol = SUM_RTOL * sums + SUM_ATOL_PER_PHOTON * count[:, None]
    assert (err <= tol).all(), f"max excess {np.max(err - tol):.3g}"
    nz = sums > 0
    strict = (err[nz] <= SUM_RTOL * sums[nz]).mean()
    assert strict >= 0.999, strict
    # the pixel image: weight x sums added per hit point
    want = np.zeros(ex["gathered"].shape, np.float64).reshape(-1, 3)
    np.add.at(want, pixel, w.astype(np.float64) * g)
    got = ex["gathered"].reshape(-1, 3).astype(np.float64)
    assert np.allclose(got, want, rtol=1e-5, atol=1e-7 * max(1.0, want.max()))
    return dict(hits=len(q), photons=len(pos), in_radius=int(count.sum()), strict=float(strict),
                max_rel=float(np.max(err[nz] / sums[nz])) if nz.any() else 0.0)


@pytest.fixture(scope="module")
def ctx():
    c = Context(0, seed=99)
    yield c
    c.close()


def _export(ctx, scene, reso, nphoton, first_pass, cells, pfilter, gather, seed=5):
    sc, cam = S.box_scene(scene), S.box_camera(reso)
    cam.pfilter = pfilter
    ctx.upload_scene(sc)
    ctx.set_camera(cam)
    ctx.render_begin(RenderConfig(nphoton=nphoton, passes=1, radius0=0.05, alpha=0.7, precision=MIXED,
                                  use_graph=False, seed=seed, first_pass=first_pass, cell_factor=cells,
                                  flags=GATHERS[gather]))
    ex = ctx.render_gather_export()
    assert ex["pass_index"] == first_pass and ex["pfilter"] == pfilter
    return ex, Oracle(sc, cam)


@pytest.mark.parametrize("gather", list(GATHERS))
@pytest.mark.parametrize("first_pass", [0, 33])
@pytest.mark.parametrize("cells", [1, 2])
def test_glass_box_render_gather_per_hit_point(ctx, gather, first_pass, cells):
    ex, orc = _export(ctx, "c2", 512, 1_000_000, first_pass, cells, S.FILTER_NONE, gather)
    r = check_export(ex, orc)
    assert r["hits"] > 262144 and r["photons"] > 500_000 and r["in_radius"] > 1e7, r


@pytest.mark.parametrize("gather", list(GATHERS))
@pytest.mark.parametrize("pfilter", [S.FILTER_CONE, S.FILTER_GAUSS])
def test_glass_box_render_gather_filters(ctx, gather, pfilter):
    ex, orc = _export(ctx, "c2", 512, 1_000_000, 33, 1, pfilter, gather)
    check_export(ex, orc)


@pytest.mark.parametrize("gather", list(GATHERS))
def test_diffuse_box_render_gather_full_size(ctx, gather):
    ex, orc = _export(ctx, "c1", 256, 200_000, 0, 1, S.FILTER_NONE, gather)
    r = check_export(ex, orc)
    assert r["hits"] > 0.9 * 65536 and r["in_radius"] > 1e6, r


def test_export_pass_counts_as_a_render_pass(ctx):
    """The export pass is one pass of the render: the running image holds it."""
    sc, cam = S.box_scene("c1"), S.box_camera(64)
    ctx.upload_scene(sc)
    ctx.set_camera(cam)
    ctx.render_begin(RenderConfig(nphoton=20000, passes=2, radius0=0.05, precision=MIXED, use_graph=True, seed=3))
    ctx.render_step(1)
    ctx.render_gather_export()
    assert ctx.stats()["passes_done"] == 2
    img = ctx.render_image()
    assert np.isfinite(img).all() and img.max() > 0

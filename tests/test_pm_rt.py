"""The pm | rt pipeline of the reference (src/bin/pm.rs, src/bin/rt.rs) on
the GPU: pm's photon map text holds exactly the oracle's photons for the
built-in scene (FP64, bit for bit after the shortest round-trip printing),
and rt's image from that text equals the oracle's eye pass over the same
photons within 1e-9."""
import subprocess

import numpy as np
import pytest

from oracle.binding import Oracle
from ppmpa_gb300 import build as lib_build, scene as S

pytestmark = pytest.mark.gpu
TOOLS = lib_build.OUT
WL = {"Red": 0, "Green": 1, "Blue": 2}


def _parse_map(text):
    lines = text.strip().split("\n")
    n, pw = int(lines[0]), float(lines[1])
    f = [l.split(" ") for l in lines[2:]]
    wl = np.array([WL[x[0]] for x in f], np.uint8)
    v = np.array([[float(t) for t in x[1:]] for x in f])
    return n, pw, wl, v[:, :3], v[:, 3:]


def test_pm_prints_the_oracle_photons_and_rt_renders_them(built_lib):
    n = 4000
    pm = subprocess.run([f"{TOOLS}/pm", "scene.scene", str(n), "--seed", "5"], capture_output=True, text=True,
                        check=True, timeout=120)
    nn, pw, wl, pos, d = _parse_map(pm.stdout)
    sc, cam = S.reference_scene(), S.reference_camera()
    orc = Oracle(sc, cam)
    o = orc.trace_photons(n, use_classic=True, seed=5, pass_index=0)
    assert nn == n and pw == o["power"]
    order = np.lexsort((-o["level"].astype(np.int64), o["emit"]))      # emission order, deepest first
    assert np.array_equal(wl, o["wl"][order])
    assert np.array_equal(pos, o["pos"][order])
    assert np.array_equal(d, o["dir"][order])

    r = 0.25
    rt = subprocess.run([f"{TOOLS}/rt", "scene.scene", "cam.scr", str(r), "--seed", "5"], input=pm.stdout,
                        capture_output=True, text=True, check=True, timeout=300)
    lines = rt.stdout.split("\n")
    assert lines[0] == "P3" and lines[3] == "256 256"
    img = np.array([[float(t) for t in l.split()] for l in lines[5:5 + 256 * 256]]).reshape(256, 256, 3)
    photons = dict(pos=pos, dir=d, wl=wl, power=pw)
    want = orc.eye_pass(photons, r * r, use_classic=True, seed=5, pass_index=0)
    assert np.allclose(img, want, rtol=1e-9, atol=1e-12 * want.max())
    assert want.max() > 0


def test_classic_tracer_matches_oracle(built_lib):
    """trace_ray_classic (the rtc binary): one FP64 pass equals the oracle's
    recursive restatement; ambient light reaches the image; rtc prints it."""
    from ppmpa_gb300 import PLAIN, MIXED, Context, RenderConfig
    from ppmpa_gb300.api import RENDER_CLASSIC
    cases = [(S.reference_scene(), S.make_camera(48, 40)),
             (S.box_scene("c2"), S.make_camera(40, 40, blur=False, ambient=(0.002, 0.001, 0.0005),
                                               eye_position=(0.0, 1.0, -2.6), target_position=(0.0, 1.0, 1.0),
                                               focus=3.6))]
    with Context(0, seed=9) as ctx:
        for sc, cam in cases:
            ctx.upload_scene(sc)
            ctx.set_camera(cam)
            got = ctx.render(RenderConfig(nphoton=1, passes=1, precision=PLAIN, seed=9, flags=RENDER_CLASSIC))
            want = Oracle(sc, cam).classic_pass(seed=9, pass_index=0)
            assert want.max() > 0
            assert np.allclose(got, want, rtol=1e-9, atol=1e-12 * want.max())
    # FP32 draws its camera jitter from 32-bit words (another sample), so
    # the precisions are compared on a camera without jitter or lens blur
    sc = S.reference_scene()
    cam = S.make_camera(48, 40, antialias=False, blur=False)
    with Context(0, seed=9) as ctx:
        ctx.upload_scene(sc)
        ctx.set_camera(cam)
        plain = ctx.render(RenderConfig(nphoton=1, passes=1, precision=PLAIN, seed=9, flags=RENDER_CLASSIC))
        mixed = ctx.render(RenderConfig(nphoton=1, passes=1, precision=MIXED, seed=9, flags=RENDER_CLASSIC))
        assert abs(mixed.mean() / plain.mean() - 1) < 1e-3
    out = subprocess.run([f"{TOOLS}/rtc", "cam.scr", "scene.scene", "--seed", "9"], capture_output=True, text=True,
                         check=True, timeout=120)
    lines = out.stdout.split("\n")
    assert lines[0] == "P3" and lines[3] == "256 256" and len(lines) >= 5 + 256 * 256

#!/usr/bin/env python
"""Throughput benchmark of the PPM-PA hot path on GB300.

A step is one progressive pass of the glass-box workload (512x512, 1M
photons per pass, glass sphere IOR 1.5 + mirror sphere, point light, r0 =
0.05, alpha = 0.7, 64 passes): emit + trace the photons, build the photon
map, trace the eye rays, gather, shrink the radius, accumulate the FP64
image.  The pass runs as one replayed CUDA graph in the mixed-precision
mode (FP32 trace/gather with Kahan flux sums, FP64 radius/average/
normalisation).  The K timed steps are passes 0..K-1 of a fresh 64-pass
render (the render's largest radii, so its slowest passes); the whole
64-pass schedule is timed as well and reported beside them.

Prints one JSON line (rank 0): metric Mphotons/s (emitted photons per
second), plus the plain FP64 path's throughput, image RMSE of both paths
against an FP64 high-pass image, the end-to-end throughput through the
public C ABI with host buffers, the roofline of the dominant kernel, the CPU
baseline (all host threads and one thread), the SM clocks sampled during the
timed region, and under "workloads" the same measurements of the other
configurations: the diffuse-sphere box (256x256, 200k photons, 10 passes),
the 1.31M-triangle mesh (1024x1024, 10M photons, 32 passes), the gather
sweep over 100M FP32 photons (uniform and clustered) and the batch of 64
uneven jobs.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                  [--workload NAME] [--workloads all|none|a,b,...]
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # glass box (glass sphere IOR 1.5 + mirror sphere), 512^2, 1M photons/pass, 64 passes
    "glass_box_512": dict(scene="c2", reso=512, nphoton=1_000_000, passes=64, r0=0.05, alpha=0.7,
                          cpu_sample_photons_1t=250_000),
    # diffuse-sphere box, 256^2, 200k photons/pass, 10 passes
    "box_256": dict(scene="c1", reso=256, nphoton=200_000, passes=10, r0=0.05, alpha=0.7),
    # box + displaced icosphere of 1,310,720 triangles (half glass), spot light,
    # 1024^2, 10M photons/pass, 32 passes; rays walk the GPU-built BVH.  The CPU
    # leg tests every object per ray as the reference does, so it times a
    # sample of photons only; no many-pass FP64 image is rendered for RMSE.
    "mesh_1024": dict(scene="mesh", mesh_level=8, reso=1024, nphoton=10_000_000, passes=32, r0=0.05, alpha=0.7,
                      rmse=False, cpu_sample_photons=64, cpu_sample_photons_1t=8, max_steps=8, plain_steps=2),
}
# gather sweep over an FP32 photon map: 100M photons, 4M queries with radii
# log-uniform over [1e-3, 2e-2] (ppmpa_gb300/workloads.py)
SWEEPS = {"gather_sweep_uniform": "uniform", "gather_sweep_clustered": "clustered"}
SWEEP_MAX_STEPS = {"uniform": 10, "clustered": 3}
# 64 seeded render jobs of uneven sizes (ppmpa_gb300/workloads.py batch_jobs),
# 8 passes each, rendered as one batch (one graph launch per pass for all jobs)
BATCHES = {"batch_64": dict(n_jobs=64, passes=8),
           # many small jobs: per-job graphs cost 20 kernel nodes each per pass
           "batch_256_small": dict(n_jobs=256, passes=8, prims=(10, 2000), reso=(48, 128),
                                   photons=(20_000, 100_000))}
# the configurations measured beside the headline, in this order
SECONDARY = ["box_256", "mesh_1024", "gather_sweep_uniform", "gather_sweep_clustered", "batch_64", "batch_256_small"]
L2_BYTES = 129 * 1024 * 1024


# Emitted photons traced through one full PA pass (trace, map build, eye pass,
# gather, accumulate), per second; the image RMSE against the FP64 many-pass
# image is reported beside it.
METRIC = "Mphotons/s per pass and image RMSE vs FP64 oracle, batched-FP32 vs plain, 1 GB300"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="glass_box_512", choices=list(WORKLOADS) + list(SWEEPS) + list(BATCHES))
    p.add_argument("--workloads", default="all",
                   help="configurations measured beside the glass-box headline: all, none or a comma list")
    p.add_argument("--sweep-photons", type=int, default=100_000_000)
    p.add_argument("--sweep-queries", type=int, default=4_000_000)
    p.add_argument("--sweep-cells", type=float, default=0.0,
                   help="FP32 map cells per radius for the sweep (0: autotune on a query sample)")
    p.add_argument("--oracle-passes", type=int, default=4096,
                   help="passes of the FP64 high-pass image the RMSE is measured against")
    p.add_argument("--no-rmse", action="store_true")
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--profile", type=int, default=0,
                   help="only run this many mixed passes (one warm-up) and exit: the profiler's command")
    p.add_argument("--precision", default="mixed", choices=["mixed", "plain"])
    p.add_argument("--cell-factor", type=int, default=0, help="grid cells per radius (0: tuned per render)")
    p.add_argument("--nphoton", type=int, default=0, help="photons per pass (0: the workload's); for profiling")
    p.add_argument("--tile-gather", action="store_true", help="mixed render: the tile gather (comparison)")
    p.add_argument("--batch-legs", default="staged,graphs,sequential",
                   help="batch workloads: which of the staged, graphs and sequential legs to run (staged always runs)")
    return p.parse_args()


def scene_of(w):
    from ppmpa_gb300 import mesh as M, scene as S
    sc = M.mesh_scene(w["mesh_level"]) if w["scene"] == "mesh" else S.box_scene(w["scene"])
    return sc, S.box_camera(w["reso"])


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def run_profile(args, w):
    from ppmpa_gb300 import MIXED, PLAIN, Context, RenderConfig
    from ppmpa_gb300.api import RENDER_TILE_GATHER
    sc, cam = scene_of(w)
    with Context(0, seed=args.seed) as ctx:
        ctx.upload_scene(sc)
        ctx.set_camera(cam)
        prec = MIXED if args.precision == "mixed" else PLAIN
        ctx.render_begin(RenderConfig(nphoton=w["nphoton"], passes=args.profile + 1, radius0=w["r0"],
                                      alpha=w["alpha"], precision=prec, use_graph=True, seed=args.seed,
                                      cell_factor=args.cell_factor,
                                      flags=RENDER_TILE_GATHER if args.tile_gather else 0))
        ctx.render_step(args.profile + 1)
        img = ctx.render_image()
        st = ctx.stats()
        # one more eager pass with the gather counters on
        ctx.set_stage_timing(2)
        ctx.render_step(1)
        ctx.sync()
        cnt = ctx.stats()
        ctx.set_stage_timing(0)
        st["stage_ms"] = cnt["stage_ms"]
        st.update({k: cnt[k] for k in ("candidates", "in_radius", "gather_slots")})
    print(json.dumps({"profile_passes": args.profile + 1, "kernels_per_pass": st["kernels_per_pass"],
                      "photons_stored": st["photons_stored"], "hit_points": st["hit_points"],
                      "grid_cells": st["grid_cells"], "candidates": st["candidates"], "in_radius": st["in_radius"],
                      "gather_slots": st["gather_slots"], "stage_ms_last": st["stage_ms"], "mean": float(img.mean())}))


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        return json.load(open(path))["hbm_gbs"], "measured"
    return 6800.0, "fallback"


def profile_summary(key):
    """Numbers from the committed ncu summaries (profiles/*.json): DRAM
    traffic per launch and instruction counts per photon test."""
    out = {}
    for name in ("traffic.json", "issue.json"):
        path = os.path.join(ROOT, "profiles", name)
        if os.path.exists(path):
            v = json.load(open(path)).get(key)
            if v is not None:
                out[name.split(".")[0]] = v
    return out


# ---------------------------------------------------------------------------
# CPU: the FP64 restatement of the reference's CPU path
# ---------------------------------------------------------------------------
def cpu_pass_rate(w, seed, threads=0, photons=None):
    """Oracle passes on `threads` host threads (0: all): photon tracing of
    `photons` (default the workload's) plus, unless the workload times
    tracing alone, the eye pass and gather over them; returns (Mphotons/s,
    threads, seconds, what)."""
    from oracle.binding import Oracle, radius_schedule
    sc, cam = scene_of(w)
    orc = Oracle(sc, cam, threads=threads)
    nth = orc.L.orc_get_threads()
    if "cpu_sample_photons" in w:      # photon tracing of a sample only
        n = photons or w["cpu_sample_photons"]
        t0 = time.perf_counter()
        orc.trace_photons(n, True, seed, 0)
        dt = time.perf_counter() - t0
        return n / dt / 1e6, nth, dt, f"photon tracing of {n} photons (every object tested per ray)"
    n = min(photons or w["nphoton"], w["nphoton"])
    r2 = radius_schedule(w["r0"], w["alpha"], 1, 1)
    t0 = time.perf_counter()
    ph = orc.trace_photons(n, True, seed, 0)
    orc.eye_pass(ph, r2[0], True, seed, 0)
    dt = time.perf_counter() - t0
    what = (f"one full pass ({n} photons, {w['reso']}x{w['reso']} eye rays)" if n == w["nphoton"] else
            f"one pass with {n} of the {w['nphoton']} photons and all {w['reso']}x{w['reso']} eye rays")
    return n / dt / 1e6, nth, dt, what


def cpu_baseline(w, seed):
    """The reference CPU path (restated) on all host threads and on one."""
    rate, threads, dt, what = cpu_pass_rate(w, seed, 0)
    r1, _, dt1, what1 = cpu_pass_rate(w, seed, 1, w.get("cpu_sample_photons_1t"))
    return {"value": rate, "unit": "Mphotons/s", "cores": threads, "kind": "port",
            "sample": f"{what}, FP64 restatement of the reference CPU path, {threads} threads, {dt:.2f} s",
            "single_thread": {"value": r1, "unit": "Mphotons/s", "cores": 1, "kind": "port",
                              "sample": f"{what1}, one thread (as the reference runs), {dt1:.2f} s"}}


def run_reference(args, w):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    for k in range(args.warmup):
        cpu_pass_rate(w, args.seed + 1000 + k)
    total = done = 0.0
    threads = 1
    what = ""
    for k in range(args.steps):
        rate, threads, dt, what = cpu_pass_rate(w, args.seed + k)
        total += dt
        done += rate * dt * 1e6                     # photons of this step's sample
    value = done / total / 1e6
    r1, _, dt1, what1 = cpu_pass_rate(w, args.seed, 1, w.get("cpu_sample_photons_1t"))
    out = {
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "Mphotons/s", "n_gpus": args.gpus, "host_only": True, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded scene, seeded photon streams)",
        "config": {"workload": args.workload, **w},
        "cpu_baseline": {"value": value, "unit": "Mphotons/s", "cores": threads, "kind": "port",
                         "sample": f"{what} per step, FP64 restatement of the reference CPU path, {threads} threads",
                         "single_thread": {"value": r1, "unit": "Mphotons/s", "cores": 1, "kind": "port",
                                           "sample": f"{what1}, one thread, {dt1:.2f} s"}},
        "e2e": {"value": value, "unit": "Mphotons/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


# ---------------------------------------------------------------------------
# GPU: progressive render workloads
# ---------------------------------------------------------------------------
def algorithmic_bytes(stage, st, npx):
    """Compulsory DRAM bytes of one launch of each stage (mixed-precision layout)."""
    nq, nph, ncell = st["hit_points"], st["photons_stored"], st["grid_cells"]
    if stage == "gather":
        # hit point (40 B) read once, 3 FP32 adds into the pass buffer, each photon
        # record (16 B) and the cell starts read once
        return nq * (40 + 12) + nph * 16 + (ncell + 1) * 4
    if stage == "photon_trace":
        return nph * 16 + nph * 16          # records written once, bounds pass reads them once
    if stage == "map_build":
        return nph * (16 + 8) + ncell * 4 * 3 + nph * (8 + 16 + 16)
    if stage == "eye_trace":
        return nq * 40 + npx * 24
    if stage == "accumulate":
        return npx * 24 * 3
    return 0


def issue_roofline(tests, gather_ms, clock_mhz, summary):
    """Instruction-issue roofline of the gather: photon tests per second times
    the warp instructions one test costs (from the committed ncu summary)
    against the SMs' issue rate (4 warp instructions per SM per cycle)."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    peak = sms * 4 * (clock_mhz or 2070.0) * 1e6
    tests_per_s = tests / (gather_ms / 1e3)
    out = {"tests_per_s": tests_per_s, "peak_warp_inst_per_s": peak, "sms": sms, "clock_mhz": clock_mhz}
    if summary and summary.get("tests"):
        wpt = summary["warp_inst"] / summary["tests"]
        out.update({"warp_inst_per_test": wpt, "thread_inst_per_test": summary["thread_inst"] / summary["tests"],
                    "achieved_warp_inst_per_s": tests_per_s * wpt, "frac": tests_per_s * wpt / peak,
                    "source": summary.get("source")})
    return out


def measure_render(args, name, w, ctx, stream, flush, world, rank, local, headline):
    """Every GPU measurement of one render workload on an open context."""
    import torch
    from ppmpa_gb300 import MIXED, PLAIN, RenderConfig
    from ppmpa_gb300.api import RENDER_TILE_GATHER, RENDER_TUNE_CELLS

    sc, cam = scene_of(w)
    ctx.upload_scene(sc)
    ctx.set_camera(cam)
    leaf = None
    if ctx.accel_info()["bvh_objects"]:
        # BVH leaf size: timed on 256k random rays through the box
        rng = np.random.default_rng(args.seed + 17)
        p = rng.uniform((-0.95, 0.05, 0.05), (0.95, 1.95, 1.95), (262144, 3))
        d = rng.normal(size=(262144, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        leaf, _ = ctx.tune_bvh_leaf(np.hstack([p, d]))
    walk = RENDER_TILE_GATHER if args.tile_gather else 0
    P = w["passes"]
    steps = min(args.steps, w.get("max_steps", args.steps))
    warmup = max(3, args.warmup) if headline else 3

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def cfg(precision, passes, first=0, graph=True, seed=None, cells=None):
        c = args.cell_factor if cells is None else cells
        return RenderConfig(nphoton=w["nphoton"], passes=passes, use_classic=True, radius0=w["r0"],
                            alpha=w["alpha"], schedule_offset=1, precision=precision, use_graph=graph,
                            seed=args.seed if seed is None else seed, first_pass=first, cell_factor=c,
                            flags=(RENDER_TUNE_CELLS if c == 0 else 0) | walk)

    def timed_passes(precision, k, seed, cells=None):
        """Warm-up render of `warmup` passes, then passes 0..k-1 of a fresh
        render of max(P, k) passes, each pass a graph replay bracketed by CUDA
        events on the library's stream, L2 flushed between passes (untimed).
        Returns (summed ms, per-pass ms list)."""
        ctx.render_begin(cfg(precision, max(P, warmup), seed=seed + 555, cells=cells))
        ctx.render_step(warmup)
        ctx.render_begin(cfg(precision, max(P, k), seed=seed, cells=cells))
        ctx.sync()
        torch.cuda.synchronize()
        barrier()
        evs = []
        for _ in range(k):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.render_step(1)
            b.record(stream)
            with torch.cuda.stream(stream):
                flush.zero_()          # evict L2 between timed passes (not timed)
            evs.append((a, b))
        torch.cuda.synchronize()
        ctx.sync()
        barrier()
        per = [a.elapsed_time(b) for a, b in evs]
        ms = sum(per)
        if world > 1:
            import torch.distributed as dist
            t = torch.tensor([ms], device=f"cuda:{local}")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms, per

    seed_rank = args.seed + 1000 * rank
    clocks = Clocks(local)
    clocks.start()
    ms, _ = timed_passes(MIXED, steps, seed_rank)
    clk = clocks.stop()
    cells = ctx.stats()["cell_factor"]
    st = ctx.stats()
    value = world * steps * w["nphoton"] / (ms / 1e3) / 1e6
    kernels_per_pass = st["kernels_per_pass"]
    # the whole schedule: all P passes of one render, timed one by one
    ms_full, per_full = timed_passes(MIXED, P, seed_rank + 9, cells=cells)
    full = {"passes": P, "ms_per_pass": ms_full / P, "value": world * P * w["nphoton"] / (ms_full / 1e3) / 1e6,
            "first_last_ms": [round(per_full[0], 4), round(per_full[-1], 4)]}

    # per-stage device time (eager passes with CUDA events between stages)
    ctx.render_begin(cfg(MIXED, max(P, steps + warmup), seed=seed_rank + 1, graph=False, cells=cells))
    ctx.render_step(warmup)
    ctx.set_stage_timing(1)
    ctx.render_step(steps)
    ctx.sync()
    st_t = ctx.stats()
    ctx.set_stage_timing(False)
    npx = w["reso"] * w["reso"]
    stage_avg = {k: st_t["stage_ms"][k] / max(1, st_t["stage_calls"][k]) for k in st_t["stage_ms"]
                 if st_t["stage_calls"][k]}
    dominant = max(stage_avg, key=stage_avg.get)
    peak, peak_src = hbm_peak()
    ab = algorithmic_bytes(dominant, st_t, npx)
    achieved = ab / (stage_avg[dominant] / 1e3) / 1e9
    # the gather's counts depend on the grid: its summaries are keyed by cells per radius
    summary = profile_summary(f"{dominant}:{name}" + (f":k{cells}" if dominant == "gather" else ""))

    stage_roof = {}
    for k, t in stage_avg.items():
        b = algorithmic_bytes(k, st_t, npx)
        if t > 0 and b > 0:
            gbs = b / (t / 1e3) / 1e9
            stage_roof[k] = {"ms": round(t, 4), "algorithmic_bytes": b, "achieved_gbs": round(gbs, 1),
                             "frac": round(gbs / peak, 4)}
    mid = P // 2                         # one pass from the middle of the render, timed, then counted
    one = cfg(MIXED, 1, first=mid, graph=False, seed=seed_rank + 4, cells=cells)
    ctx.render_begin(one)
    before = ctx.stats()["stage_ms"]["gather"]
    ctx.set_stage_timing(1)
    ctx.render_step(1)
    ctx.sync()
    g_ms = ctx.stats()["stage_ms"]["gather"] - before
    ctx.render_begin(one)
    ctx.set_stage_timing(2)
    ctx.render_step(1)
    ctx.sync()
    cnt = ctx.stats()
    ctx.set_stage_timing(False)
    rates = {
        "photon_rays_per_s": st_t["photon_rays"] / (stage_avg["photon_trace"] / 1e3),
        "eye_rays_per_s": st_t["eye_rays"] / (stage_avg["eye_trace"] / 1e3),
        "photon_rays_per_pass": st_t["photon_rays"], "eye_rays_per_pass": st_t["eye_rays"],
        "photon_tests_per_s": cnt["candidates"] / (g_ms / 1e3), "in_radius_per_s": cnt["in_radius"] / (g_ms / 1e3),
        "photon_tests": cnt["candidates"], "in_radius": cnt["in_radius"], "lane_slots": cnt["gather_slots"],
        "tests_per_in_radius": cnt["candidates"] / max(1, cnt["in_radius"]),
        "gather_ms": round(g_ms, 4),
        "pass": mid,
        "note": ("ray rates: last pass of the stage-timed run over its stage's mean time (eye rays: primary "
                 "and reflected/refracted children, shadow rays not counted); photon tests: one pass from the "
                 "middle of the render, timed, then replayed with the gather counters on"),
    }
    roofline = {"kernel": dominant, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": summary.get("traffic"), "peak_source": peak_src,
                "algorithmic_bytes": ab}
    if dominant == "gather":
        roofline["issue"] = issue_roofline(cnt["candidates"], g_ms, clk.get("sm_mhz"), summary.get("issue"))
        roofline["note"] = ("the gather keeps the photon map and hit points in L2 and is bound by instruction "
                            "issue; the HBM fraction is secondary, the issue block is the bound")

    # plain FP64 path on the same workload
    steps_plain = w.get("plain_steps", max(3, min(steps, 10)))
    ms_plain, _ = timed_passes(PLAIN, steps_plain, seed_rank + 2, cells=cells)
    value_plain = world * steps_plain * w["nphoton"] / (ms_plain / 1e3) / 1e6

    out_rmse = None
    if not args.no_rmse and w.get("rmse", True) and rank == 0:
        # The FP32 and FP64 paths draw from different random streams (the FP32
        # emission samples the sphere directly), so their errors are
        # independent noise: each precision's RMSE is the mean over two seeds.
        t0 = time.perf_counter()
        ctx.render_begin(cfg(PLAIN, args.oracle_passes, seed=args.seed + 7919, cells=cells))
        ctx.render_step(args.oracle_passes)
        img_ref = ctx.render_image()
        t_oracle = time.perf_counter() - t0
        errs = {MIXED: [], PLAIN: []}
        for k in range(2):
            for prec in (MIXED, PLAIN):
                ctx.render_begin(cfg(prec, P, seed=seed_rank + 10 * k, cells=cells))
                ctx.render_step(P)
                errs[prec].append(float(np.sqrt(np.mean((ctx.render_image() - img_ref) ** 2))))
        rm, rp = float(np.mean(errs[MIXED])), float(np.mean(errs[PLAIN]))
        out_rmse = {"mixed": rm, "plain": rp, "mixed_over_plain": rm / rp, "passes": P, "seeds": 2,
                    "per_seed": {"mixed": errs[MIXED], "plain": errs[PLAIN]},
                    "oracle": f"FP64 plain GPU path, {args.oracle_passes} passes, independent seed",
                    "oracle_seconds": round(t_oracle, 2), "mean_radiance": float(img_ref.mean())}

    # end to end through the public C ABI: scene + camera upload, a full
    # progressive render, image download (host buffers), per step
    e2e_steps = 3 if headline else 1
    ctx.sync()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        ctx.upload_scene(sc)
        ctx.set_camera(cam)
        img = ctx.render(cfg(MIXED, P, seed=seed_rank + 3 + k, cells=cells))
    t_e2e = time.perf_counter() - t0
    e2e_value = world * e2e_steps * P * w["nphoton"] / t_e2e / 1e6
    import ctypes
    from ppmpa_gb300 import scene as S
    h2d = (ctypes.sizeof(S.Object) * sc.n_objects + ctypes.sizeof(S.Material) * len(sc.materials) +
           ctypes.sizeof(S.Light) * len(sc.lights) + ctypes.sizeof(S.Camera))
    d2h = img.nbytes

    cpu = cpu_baseline(w, args.seed) if rank == 0 else None
    return {
        "value": value, "unit": "Mphotons/s", "steps": steps, "warmup": warmup, "ms_per_step": ms / steps,
        "config": {"workload": name, **{k: v for k, v in w.items() if not k.startswith("cpu_")},
                   "precision": "mixed", "cuda_graph": True, "bvh_leaf": leaf, "cells_per_radius": cells,
                   "gather": "tile" if args.tile_gather else "row walk",
                   "timed_passes": [0, steps - 1], "schedule_passes": max(P, steps),
                   "l2": "flushed between timed passes (2x L2 write)", "parallelism": f"passes x{world}"},
        "full_schedule": full,
        "plain_fp64": {"value": value_plain, "unit": "Mphotons/s", "ms_per_step": ms_plain / steps_plain,
                       "steps": steps_plain, "mixed_over_plain": value / value_plain},
        "rmse": out_rmse,
        "e2e": {"value": e2e_value, "unit": "Mphotons/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "step": f"ppm_scene_upload + ppm_camera_set + ppm_render({P} passes, cell size {cells} "
                        f"as tuned above) + image download"},
        "gpu_launches": kernels_per_pass * steps,
        "kernels_per_pass": kernels_per_pass,
        "stages_ms_per_pass": {k: round(v, 4) for k, v in stage_avg.items()},
        "roofline": roofline,
        "stage_rooflines": stage_roof,
        "rates": rates,
        "pass_stats": {"photons_stored": st["photons_stored"], "hit_points": st["hit_points"],
                       "grid_cells": st["grid_cells"]},
        "cpu_baseline": cpu,
        "clocks": clk,
    }


def run_gpu(args, w):
    import torch
    from ppmpa_gb300 import Context

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}")
    ctx = Context(local, seed=args.seed)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    r = measure_render(args, args.workload, w, ctx, stream, flush, world, rank, local, headline=True)
    ctx.close()
    if rank != 0:
        return
    out = {
        "metric": METRIC, "value": r["value"], "unit": "Mphotons/s", "n_gpus": world, "steps": r["steps"],
        "warmup": r["warmup"], "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 trace/gather, f64 radius/average",
        "data": "synthetic (seeded scene, seeded photon streams)",
    }
    out.update({k: v for k, v in r.items() if k not in out})
    names = SECONDARY if args.workloads == "all" else [] if args.workloads == "none" else args.workloads.split(",")
    if args.workload == "glass_box_512" and names:
        out["workloads"] = run_secondary(args, names, flush, stream_local=local)
    print(json.dumps(out), flush=True)


def run_secondary(args, names, flush, stream_local):
    """The other configurations, each on a fresh context: a failure is
    recorded in its entry and does not stop the others."""
    import torch
    from ppmpa_gb300 import Context
    out = {}
    for name in names:
        t0 = time.perf_counter()
        try:
            if name in WORKLOADS:
                ctx = Context(stream_local, seed=args.seed)
                stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", stream_local))
                try:
                    r = measure_render(args, name, WORKLOADS[name], ctx, stream, flush, 1, 0, stream_local,
                                       headline=False)
                finally:
                    ctx.close()
            elif name in SWEEPS:
                r = measure_sweep(args, name, SWEEPS[name])
            elif name in BATCHES:
                r = measure_batch(args, name, BATCHES[name])
            else:
                r = {"error": f"unknown workload {name}"}
        except Exception as e:   # noqa: BLE001 -- recorded, the rest still run
            r = {"error": f"{type(e).__name__}: {e}"}
        r["wall_s"] = round(time.perf_counter() - t0, 1)
        out[name] = r
        torch.cuda.empty_cache()
    return out


# ---------------------------------------------------------------------------
# GPU: the gather sweep over an FP32 photon map
# ---------------------------------------------------------------------------
def sweep_inputs(args, kind):
    from ppmpa_gb300 import workloads as W
    pos, d, wl = W.photons(args.sweep_photons, kind)
    q, nrm, r2 = W.queries(args.sweep_queries, kind)
    return pos, d, wl, q, nrm, r2


def measure_sweep(args, name, kind, inputs=None):
    """One step = one ppm_estimate_f32 call over all queries (host arrays in,
    host results out).  value: estimates per second of the device work (query
    sort + gather); e2e: the same through the call with its copies."""
    from ppmpa_gb300 import Context, workloads as W
    t0 = time.perf_counter()
    pos, d, wl, q, nrm, r2 = inputs or sweep_inputs(args, kind)
    gen_s = time.perf_counter() - t0
    n_ph, n_q = len(pos), len(q)
    steps = min(args.steps, SWEEP_MAX_STEPS[kind])
    ctx = Context(0, seed=args.seed)
    ctx.set_stage_timing(1)
    ctx.build_photonmap_f32(pos, d, wl, 1.0 / n_ph, W.R_MAX ** 2)
    ctx.build_photonmap_f32(pos, d, wl, 1.0 / n_ph, W.R_MAX ** 2)   # second build: warm
    build_ms = ctx.stats()["stage_ms"]["map_build"] / 2
    if args.sweep_cells > 0:
        ctx.regrid_photonmap_f32(args.sweep_cells)
        cells, tune = args.sweep_cells, None
    else:
        sub = np.random.default_rng(11).choice(n_q, min(n_q, 262144), replace=False)
        cells, tune_ms = ctx.tune_photonmap_f32(q[sub], nrm[sub], r2[sub])
        tune = {"sample_queries": len(sub), "best_ms": tune_ms}
    ctx.set_stage_timing(2)                         # one counted run: candidates and hits
    ctx.estimate_f32(q, nrm, r2)
    cnt = ctx.stats()
    ctx.set_stage_timing(1)
    for _ in range(3):
        ctx.estimate_f32(q, nrm, r2)
    base = ctx.stats()
    clocks = Clocks(0)
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(steps):
        ctx.estimate_f32(q, nrm, r2)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    st = ctx.stats()
    ctx.close()
    gather_ms = (st["stage_ms"]["gather"] - base["stage_ms"]["gather"]) / steps
    sort_ms = (st["stage_ms"]["query_sort"] - base["stage_ms"]["query_sort"]) / steps
    dev_ms = gather_ms + sort_ms
    peak, src = hbm_peak()
    photon_bytes = 16                               # float3 position + packed direction/wavelength
    query_bytes = 12 + 12 + 8 + 24                  # position, normal, radius^2 in; RGB out
    ab = n_ph * photon_bytes + n_q * query_bytes
    achieved = ab / (gather_ms / 1e3) / 1e9
    summary = profile_summary(name)
    cpu = cpu_sweep(pos, d, wl, q, nrm, r2)
    return {
        "metric": f"gather sweep estimates/s ({n_ph} FP32 photons, {n_q} queries, r log-uniform 1e-3..2e-2)",
        "value": n_q / (dev_ms / 1e3) / 1e6, "unit": "Mqueries/s", "steps": steps,
        "warmup": 3, "ms_per_step": dev_ms, "higher_is_better": True,
        "dtype": "f32 positions/tests, f64 rounding-band recheck and normalisation",
        "data": "synthetic (seeded photons and queries)",
        "config": {"workload": name, "distribution": kind, "photons": n_ph, "queries": n_q,
                   "r_min": W.R_MIN, "r_max": W.R_MAX, "cells_per_radius": cells, "autotune": tune,
                   "l2": f"inputs larger than L2 (map {n_ph * photon_bytes / 2**30:.2f} GiB)"},
        "gather_ms": gather_ms, "query_sort_ms": sort_ms, "map_build_ms": build_ms,
        "photon_tests_per_s": cnt["candidates"] / (gather_ms / 1e3), "in_radius_per_s": cnt["in_radius"] / (gather_ms / 1e3),
        "candidates": cnt["candidates"], "in_radius": cnt["in_radius"], "lane_slots": cnt["gather_slots"],
        "e2e": {"value": n_q * steps / wall / 1e6, "unit": "Mqueries/s",
                "h2d_bytes_per_step": n_q * (12 + 12 + 8), "d2h_bytes_per_step": n_q * 24,
                "step": "ppm_estimate_f32 over all queries, pageable host arrays"},
        "gpu_launches": 6 * steps,
        "roofline": {"kernel": "gather", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": summary.get("traffic"), "peak_source": src,
                     "algorithmic_bytes": ab},
        "cpu_baseline": cpu,
        "input_generation_s": gen_s, "clocks": clk,
    }


def cpu_sweep(pos, d, wl, q, nrm, r2, n_all=20000, n_one=2000, steps=1):
    """The FP64 restatement of the reference's estimate (grid in place of the
    kd-tree) over the full map, on a bounded sample of the queries, on all
    host threads and on one."""
    from oracle.binding import Oracle
    from ppmpa_gb300 import scene as S
    p64, d64 = pos.astype(np.float64), d.astype(np.float64)
    res = {}
    for threads, n_s in ((0, n_all), (1, n_one)):
        orc = Oracle(S.Scene(), threads=threads)
        nth = orc.L.orc_get_threads()
        n_s = min(len(q), n_s)
        qs, ns, rs = q[:n_s].astype(np.float64), nrm[:n_s].astype(np.float64), r2[:n_s]
        total = 0.0
        for _ in range(steps):
            orc.estimate_radii(p64, d64, wl, qs, ns, rs, 1.0 / len(pos))
            total += orc.L.orc_last_query_seconds()   # query phase; the grid build is not timed
        res[threads] = (n_s * steps / total / 1e6, nth, n_s, total)
    v, nth, n_s, t = res[0]
    v1, _, n1, t1 = res[1]
    return {"value": v, "unit": "Mqueries/s", "cores": nth, "kind": "port",
            "sample": f"{n_s} of the queries over the full map, {nth} threads, grid build excluded, {t:.2f} s",
            "single_thread": {"value": v1, "unit": "Mqueries/s", "cores": 1, "kind": "port",
                              "sample": f"{n1} of the queries, one thread, {t1:.2f} s"}}


def run_sweep_reference(args, kind):
    """The FP64 restatement of the reference's estimate over the same map, on a
    bounded sample of the queries per step."""
    pos, d, wl, q, nrm, r2 = sweep_inputs(args, kind)
    cpu = cpu_sweep(pos, d, wl, q, nrm, r2, steps=max(1, args.steps // 5))
    value = cpu["value"]
    print(json.dumps({
        "impl": "reference", "metric": f"gather sweep estimates/s ({len(pos)} FP32 photons, {len(q)} queries, "
                                       f"r log-uniform 1e-3..2e-2)",
        "value": value, "unit": "Mqueries/s", "n_gpus": args.gpus, "host_only": True, "steps": args.steps,
        "warmup": max(1, args.warmup), "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded photons and queries)",
        "config": {"workload": args.workload, "distribution": kind, "photons": len(pos), "queries": len(q)},
        "cpu_baseline": cpu,
        "e2e": {"value": value, "unit": "Mqueries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


# ---------------------------------------------------------------------------
# GPU: the batch of uneven jobs
# ---------------------------------------------------------------------------
def measure_batch(args, name, bw):
    """A step = one pass of every job.  value: photons of all jobs per second
    of batch device time, in the mode PPM_BATCH_AUTO picked (its trial, on
    the warm-up render, times one pass of staged passes and one of the jobs'
    graphs side by side, and keeps the faster); the other mode and the jobs
    rendered one after another are timed beside it; e2e: Batch.render wall
    time (scene uploads, BVH builds, cell tuning, graph capture, passes,
    images)."""
    import torch
    from ppmpa_gb300 import Batch, Context, workloads as W
    from ppmpa_gb300.api import BATCH_AUTO, BATCH_GRAPHS, BATCH_STAGED
    jobs = W.batch_jobs(bw["n_jobs"], seed=args.seed + 6, passes=bw["passes"],
                        **{k: bw[k] for k in ("prims", "reso", "photons") if k in bw})
    photons = sum(cfg.nphoton for _, _, cfg in jobs) * bw["passes"]
    legs = args.batch_legs.split(",")
    with Batch(0, seed=args.seed) as b:
        b.set_mode(BATCH_AUTO)
        b.render(jobs)                                   # warm-up: allocations, module loads, AUTO's trial
        info = b.info()
        picked = "staged" if info["staged"] else "graphs"
        clocks = Clocks(0)
        clocks.start()
        t0 = time.perf_counter()
        imgs, dev_ms = b.render(jobs)                    # AUTO keeps its pick
        wall = time.perf_counter() - t0
        clk = clocks.stop()
        mode_ms = {picked: dev_ms}
        if "staged" in legs and picked != "staged":
            b.set_mode(BATCH_STAGED, info["tile"])
            b.render(jobs)
            _, mode_ms["staged"] = b.render(jobs)
        if "graphs" in legs and picked != "graphs":
            b.set_mode(BATCH_GRAPHS)
            b.render(jobs)
            _, mode_ms["graphs"] = b.render(jobs)
    seq_ms = None if "sequential" not in legs else 0.0
    with Context(0, seed=args.seed) as ctx:
        for sc, cam, cfg in (jobs if seq_ms is not None else []):
            ctx.upload_scene(sc)
            ctx.set_camera(cam)
            ctx.render_begin(cfg)
            ctx.sync()
            a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            st = torch.cuda.ExternalStream(ctx.stream)
            a.record(st)
            ctx.render_step(cfg.passes)
            e.record(st)
            ctx.sync()
            torch.cuda.synchronize()
            seq_ms += a.elapsed_time(e)
    prims = [sc.n_objects for sc, _, _ in jobs]

    def rate(ms):
        return None if ms is None else {"value": photons / (ms / 1e3) / 1e6, "unit": "Mphotons/s", "ms": ms}
    # kernels of this library launched in the timed render: 22 per staged pass
    # of the batch, or each job's pass graph per pass inside the parent graphs
    # (20 kernels, 22 when its scene holds an infinite plane: the photon bounds
    # and the grid set-up, which the photon trace does for bounded scenes)
    def per_pass(sc):
        from ppmpa_gb300 import scene as S
        plane = any(sh.shape == S.SHAPE_PLAIN for sh, _ in sc.objects) or \
            any(bool((b["shape"] == S.SHAPE_PLAIN).any()) for b in sc.bulk)
        return 22 if plane else 20
    launches = 22 * bw["passes"] if picked == "staged" else sum(per_pass(sc) * cfg.passes for sc, _, cfg in jobs)
    return {
        "metric": f"batched render Mphotons/s ({len(jobs)} uneven jobs, all passes of every job)",
        "value": photons / (dev_ms / 1e3) / 1e6, "unit": "Mphotons/s", "steps": bw["passes"],
        "warmup": 1, "ms_per_step": dev_ms / bw["passes"], "higher_is_better": True,
        "dtype": "f32 trace/gather, f64 radius/average", "data": "synthetic (seeded scenes)",
        "config": {"workload": name, "jobs": len(jobs), "passes": bw["passes"],
                   "primitives": [min(prims), max(prims), sum(prims)],
                   "photons_per_pass": [min(c.nphoton for _, _, c in jobs), max(c.nphoton for _, _, c in jobs)],
                   "reso": [min(c.xreso for _, c, _ in jobs), max(c.xreso for _, c, _ in jobs)],
                   "cell_tuning": True, "mode": picked, "staged_tile": info["tile"],
                   "auto_trial_ms_per_pass": info.get("trial_ms")},
        "staged": rate(mode_ms.get("staged")),
        "graphs": dict(rate(mode_ms.get("graphs")) or {},
                       note="each job's pass graph, all jobs' graphs in one parent graph per pass")
        if mode_ms.get("graphs") is not None else None,
        "staged_over_graphs": (mode_ms["graphs"] / mode_ms["staged"]
                               if mode_ms.get("staged") and mode_ms.get("graphs") else None),
        "gpu_launches": launches,
        "sequential": rate(seq_ms),
        "batch_over_sequential": None if seq_ms is None else seq_ms / dev_ms,
        "e2e": {"value": photons / wall / 1e6, "unit": "Mphotons/s",
                "h2d_bytes_per_step": sum(120 * sc.n_objects + 168 * len(sc.materials) + 160 * len(sc.lights) + 336
                                          for sc, _, _ in jobs),
                "d2h_bytes_per_step": sum(i.nbytes for i in imgs),
                "step": "Batch.render: uploads, BVH builds, cell tuning, capture, all passes, images"},
        "cpu_baseline": None,
        "cpu_baseline_note": ("no CPU leg: the reference tests every object per ray and renders one scene per "
                              "process; the per-configuration CPU rates are under box_256 and mesh_1024"),
        "nonfinite_pixels": int(sum(int((~np.isfinite(i)).any(axis=-1).sum()) for i in imgs)),
        "mean_radiance": float(np.mean([np.nanmean(i) for i in imgs])), "clocks": clk,
    }


def main():
    args = parse()
    rank = dist_env()[0]
    if args.workload in BATCHES:
        if rank == 0 and args.impl != "reference":
            r = measure_batch(args, args.workload, BATCHES[args.workload])
            print(json.dumps({"n_gpus": 1, "scaling": "weak", "vs_baseline": None, **r}), flush=True)
        elif rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the batch workload has no CPU leg: the reference "
                              "tests every object per ray and renders one scene per process"}))
        return
    if args.nphoton > 0 and args.workload in WORKLOADS:
        WORKLOADS[args.workload] = dict(WORKLOADS[args.workload], nphoton=args.nphoton)
    if args.workload in SWEEPS:
        if rank == 0:
            if args.impl == "reference":
                run_sweep_reference(args, SWEEPS[args.workload])
            else:
                r = measure_sweep(args, args.workload, SWEEPS[args.workload])
                print(json.dumps({"n_gpus": 1, "scaling": "weak", "vs_baseline": None, **r}), flush=True)
        return
    w = WORKLOADS[args.workload]
    if args.profile:
        run_profile(args, w)
    elif args.impl == "reference":
        run_reference(args, w)
    else:
        run_gpu(args, w)


if __name__ == "__main__":
    main()

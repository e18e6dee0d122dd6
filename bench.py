#!/usr/bin/env python
"""Throughput benchmark of the PPM-PA hot path on GB300.

A step is one progressive pass of the glass-box workload (512x512, 1M
photons per pass, glass sphere IOR 1.5 + mirror sphere, point light, r0 =
0.05, alpha = 0.7): emit + trace the photons, build the photon map, trace
the eye rays, gather, shrink the radius, accumulate the FP64 image.  The
pass runs as one replayed CUDA graph in the mixed-precision mode (FP32
trace/gather with Kahan flux sums, FP64 radius/average/normalisation).

Prints one JSON line (rank 0): metric Mphotons/s (emitted photons per
second), plus the plain FP64 path's throughput, image RMSE of both paths
against an FP64 high-pass image, the end-to-end throughput through the
public C ABI with host buffers, the roofline of the dominant kernel, the CPU
baseline and the SM clocks sampled during the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
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
    "glass_box_512": dict(scene="c2", reso=512, nphoton=1_000_000, passes=64, r0=0.05, alpha=0.7),
    # diffuse-sphere box, 256^2, 200k photons/pass, 10 passes
    "box_256": dict(scene="c1", reso=256, nphoton=200_000, passes=10, r0=0.05, alpha=0.7),
    # box + displaced icosphere of 1,310,720 triangles (half glass), spot light,
    # 1024^2, 10M photons/pass, 32 passes; rays walk the GPU-built BVH.  The CPU
    # leg tests every object per ray as the reference does, so it times a
    # sample of photons only; no many-pass FP64 image is rendered for RMSE.
    "mesh_1024": dict(scene="mesh", mesh_level=8, reso=1024, nphoton=10_000_000, passes=32, r0=0.05, alpha=0.7,
                      rmse=False, cpu_sample_photons=256),
}
# gather sweep over an FP32 photon map: 100M photons, 4M queries with radii
# log-uniform over [1e-3, 2e-2] (ppmpa_gb300/workloads.py)
SWEEPS = {"gather_sweep_uniform": "uniform", "gather_sweep_clustered": "clustered"}
# 64 seeded render jobs of uneven sizes (ppmpa_gb300/workloads.py batch_jobs),
# 8 passes each, rendered as one batch (one graph launch per pass for all jobs)
BATCHES = {"batch_64": dict(n_jobs=64, passes=8)}
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
    return p.parse_args()


def run_profile(args, w):
    from ppmpa_gb300 import MIXED, PLAIN, Context, RenderConfig
    sc, cam = scene_of(w)
    with Context(0, seed=args.seed) as ctx:
        ctx.upload_scene(sc)
        ctx.set_camera(cam)
        prec = MIXED if args.precision == "mixed" else PLAIN
        ctx.render_begin(RenderConfig(nphoton=w["nphoton"], passes=args.profile + 1, radius0=w["r0"],
                                      alpha=w["alpha"], precision=prec, use_graph=True, seed=args.seed,
                                      cell_factor=args.cell_factor))
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


def scene_of(w):
    from ppmpa_gb300 import mesh as M, scene as S
    sc = M.mesh_scene(w["mesh_level"]) if w["scene"] == "mesh" else S.box_scene(w["scene"])
    return sc, S.box_camera(w["reso"])


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


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


# ---------------------------------------------------------------------------
# CPU: the FP64 restatement of the reference's CPU path
# ---------------------------------------------------------------------------
def cpu_pass_rate(w, seed, passes=1):
    """Oracle passes (trace + eye/gather) on all host threads; returns (Mphotons/s, threads, seconds)."""
    from oracle.binding import Oracle, radius_schedule
    sc, cam = scene_of(w)
    orc = Oracle(sc, cam, threads=0)
    if "cpu_sample_photons" in w:      # photon tracing of a sample only
        n = w["cpu_sample_photons"]
        t0 = time.perf_counter()
        orc.trace_photons(n, True, seed, 0)
        dt = time.perf_counter() - t0
        return n / dt / 1e6, orc.L.orc_get_threads(), dt
    r2 = radius_schedule(w["r0"], w["alpha"], 1, passes)
    img = np.zeros((cam.yreso, cam.xreso, 3))
    t0 = time.perf_counter()
    for k in range(passes):
        ph = orc.trace_photons(w["nphoton"], True, seed, k)
        img += orc.eye_pass(ph, r2[k], True, seed, k)
    dt = time.perf_counter() - t0
    return w["nphoton"] * passes / dt / 1e6, orc.L.orc_get_threads(), dt


def run_reference(args, w):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    for k in range(args.warmup):
        cpu_pass_rate(w, args.seed + 1000 + k)
    total = done = 0.0
    threads = 1
    for k in range(args.steps):
        rate, threads, dt = cpu_pass_rate(w, args.seed + k)
        total += dt
        done += rate * dt * 1e6                     # photons of this step's sample
    value = done / total / 1e6
    what = (f"photon tracing of {w['cpu_sample_photons']} photons per step (every object tested per ray)"
            if "cpu_sample_photons" in w else
            f"one full pass per step ({w['nphoton']} photons, {w['reso']}x{w['reso']} eye rays)")
    out = {
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "Mphotons/s", "n_gpus": args.gpus, "host_only": True, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded scene, seeded photon streams)",
        "config": {"workload": args.workload, **w},
        "cpu_baseline": {"value": value, "unit": "Mphotons/s", "cores": threads, "kind": "port",
                         "sample": f"{what}, FP64 restatement of the reference CPU path, {threads} threads"},
        "e2e": {"value": value, "unit": "Mphotons/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def algorithmic_bytes(stage, st, npx):
    """Compulsory DRAM bytes of one launch of each stage (mixed-precision layout)."""
    nq, nph, ncell = st["hit_points"], st["photons_stored"], st["grid_cells"]
    if stage == "gather":
        # hit point (40 B) read once, 3 FP64 adds into the pass image, each photon
        # record (16 B) and the cell starts read once
        return nq * (40 + 48) + nph * 16 + (ncell + 1) * 4
    if stage == "photon_trace":
        return nph * 16 + nph * 16          # records written once, bounds pass reads them once
    if stage == "map_build":
        return nph * (16 + 8) + ncell * 4 * 3 + nph * (8 + 16 + 16)
    if stage == "eye_trace":
        return nq * 40 + npx * 24
    if stage == "accumulate":
        return npx * 24 * 3
    return 0


def run_gpu(args, w):
    import torch
    from ppmpa_gb300 import MIXED, PLAIN, Context, RenderConfig

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    sc, cam = scene_of(w)
    ctx = Context(local, seed=args.seed)
    ctx.upload_scene(sc)
    ctx.set_camera(cam)
    leaf = None
    if ctx.accel_info()["bvh_objects"]:
        # BVH leaf size: timed on 256k random rays through the box
        rng = np.random.default_rng(args.seed + 17)
        p = rng.uniform((-0.95, 0.05, 0.05), (0.95, 1.95, 1.95), (262144, 3))
        d = rng.normal(size=(262144, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        leaf, leaf_ms = ctx.tune_bvh_leaf(np.hstack([p, d]))
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}")

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def cfg(precision, passes, first=0, graph=True, seed=None):
        return RenderConfig(nphoton=w["nphoton"], passes=passes, use_classic=True, radius0=w["r0"],
                            alpha=w["alpha"], schedule_offset=1, precision=precision, use_graph=graph,
                            seed=args.seed if seed is None else seed, first_pass=first, cell_factor=args.cell_factor,
                            flags=1 if args.cell_factor == 0 else 0)   # 1: cell-size autotuner

    def timed_passes(precision, steps, warmup, seed):
        ctx.render_begin(cfg(precision, steps + warmup, seed=seed))
        ctx.render_step(warmup)
        ctx.sync()
        torch.cuda.synchronize()
        barrier()
        evs = []
        for _ in range(steps):
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
        ms = sum(a.elapsed_time(b) for a, b in evs)
        if world > 1:
            import torch.distributed as dist
            t = torch.tensor([ms], device=f"cuda:{local}")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    # every run renders passes from pass 0 (the PA radius schedule starts
    # there); independent random streams come from distinct seeds
    seed_rank = args.seed + 1000 * rank
    clocks = Clocks(local)
    clocks.start()
    ms = timed_passes(MIXED, args.steps, max(3, args.warmup), seed_rank)
    cells = ctx.stats()["cell_factor"]
    clk = clocks.stop()
    st = ctx.stats()
    value = world * args.steps * w["nphoton"] / (ms / 1e3) / 1e6
    kernels_per_pass = st["kernels_per_pass"]

    # per-stage device time (eager passes with CUDA events between stages)
    ctx.render_begin(cfg(MIXED, args.steps + max(3, args.warmup), seed=seed_rank + 1, graph=False))
    ctx.render_step(max(3, args.warmup))
    ctx.set_stage_timing(1)
    ctx.render_step(args.steps)
    ctx.sync()
    st_t = ctx.stats()
    ctx.set_stage_timing(False)
    npx = w["reso"] * w["reso"]
    stage_avg = {k: st_t["stage_ms"][k] / max(1, st_t["stage_calls"][k]) for k in st_t["stage_ms"]}
    dominant = max(stage_avg, key=stage_avg.get)
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak, peak_src = json.load(open(peaks_path))["hbm_gbs"], "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    ab = algorithmic_bytes(dominant, st_t, npx)
    achieved = ab / (stage_avg[dominant] / 1e3) / 1e9
    traffic = None
    prof_sum = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(prof_sum):
        traffic = json.load(open(prof_sum)).get(dominant)

    # throughput of each stage: rays, photon tests and compulsory bytes per second
    stage_roof = {}
    for k, t in stage_avg.items():
        b = algorithmic_bytes(k, st_t, npx)
        if t > 0 and b > 0:
            gbs = b / (t / 1e3) / 1e9
            stage_roof[k] = {"ms": round(t, 4), "algorithmic_bytes": b, "achieved_gbs": round(gbs, 1),
                             "frac": round(gbs / peak, 4)}
    mid = w["passes"] // 2                         # one pass from the middle of the render, timed, then counted
    one = cfg(MIXED, 1, first=mid, graph=False, seed=seed_rank + 4)
    one.cell_factor, one.flags = cells, 0
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
        "candidates": cnt["candidates"], "in_radius": cnt["in_radius"], "lane_slots": cnt["gather_slots"],
        "gather_ms": round(g_ms, 4),
        "pass": mid + 1,
        "note": ("ray rates: last pass of the stage-timed run over its stage's mean time (eye rays: primary "
                 "and reflected/refracted children, shadow rays not counted); photon tests: one pass from the "
                 "middle of the render, timed, then replayed with the gather counters on"),
    }

    # plain FP64 path on the same workload
    steps_plain = max(3, min(args.steps, 10))
    ms_plain = timed_passes(PLAIN, steps_plain, 3, seed_rank + 2)
    value_plain = world * steps_plain * w["nphoton"] / (ms_plain / 1e3) / 1e6

    out_rmse = None
    if not args.no_rmse and w.get("rmse", True) and rank == 0:
        # The FP32 and FP64 paths draw from different random streams (the FP32
        # emission samples the sphere directly), so their errors are
        # independent noise: each precision's RMSE is the mean over two seeds.
        P = w["passes"]
        t0 = time.perf_counter()
        ctx.render_begin(cfg(PLAIN, args.oracle_passes, seed=args.seed + 7919))
        ctx.render_step(args.oracle_passes)
        img_ref = ctx.render_image()
        t_oracle = time.perf_counter() - t0
        errs = {MIXED: [], PLAIN: []}
        for k in range(2):
            for prec in (MIXED, PLAIN):
                ctx.render_begin(cfg(prec, P, seed=seed_rank + 10 * k))
                ctx.render_step(P)
                errs[prec].append(float(np.sqrt(np.mean((ctx.render_image() - img_ref) ** 2))))
        rm, rp = float(np.mean(errs[MIXED])), float(np.mean(errs[PLAIN]))
        out_rmse = {"mixed": rm, "plain": rp, "mixed_over_plain": rm / rp, "passes": P, "seeds": 2,
                    "per_seed": {"mixed": errs[MIXED], "plain": errs[PLAIN]},
                    "oracle": f"FP64 plain GPU path, {args.oracle_passes} passes, independent seed",
                    "oracle_seconds": round(t_oracle, 2), "mean_radiance": float(img_ref.mean())}

    # end to end through the public C ABI: scene + camera upload, a full
    # progressive render, image download (host buffers), per step
    e2e_steps = 3
    ctx.sync()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        ctx.upload_scene(sc)
        ctx.set_camera(cam)
        c = cfg(MIXED, w["passes"], seed=seed_rank + 3 + k)
        c.cell_factor, c.flags = cells, 0          # the cell size tuned above, as a repeat caller passes it
        img = ctx.render(c)
    t_e2e = time.perf_counter() - t0
    e2e_value = world * e2e_steps * w["passes"] * w["nphoton"] / t_e2e / 1e6
    import ctypes
    from ppmpa_gb300 import scene as S
    h2d = (ctypes.sizeof(S.Object) * sc.n_objects + ctypes.sizeof(S.Material) * len(sc.materials) +
           ctypes.sizeof(S.Light) * len(sc.lights) + ctypes.sizeof(S.Camera))
    d2h = img.nbytes

    cpu = None
    if rank == 0:
        rate, threads, dt = cpu_pass_rate(w, args.seed, 1)
        what = (f"photon tracing of {w['cpu_sample_photons']} photons (every object tested per ray)"
                if "cpu_sample_photons" in w else f"one full pass ({w['nphoton']} photons, {w['reso']}x{w['reso']})")
        cpu = {"value": rate, "unit": "Mphotons/s", "cores": threads, "kind": "port",
               "sample": f"{what}, FP64 restatement of the reference CPU path, {threads} threads, {dt:.2f} s"}

    ctx.close()
    if rank != 0:
        return
    out = {
        "metric": METRIC,
        "value": value, "unit": "Mphotons/s", "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup),
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 trace/gather, f64 radius/average", "data": "synthetic (seeded scene, seeded photon streams)",
        "config": {"workload": args.workload, **w, "precision": "mixed", "cuda_graph": True, "bvh_leaf": leaf,
                   "cells_per_radius": cells,
                   "l2": "flushed between timed passes (2x L2 write)", "parallelism": f"passes x{world}"},
        "plain_fp64": {"value": value_plain, "unit": "Mphotons/s", "ms_per_step": ms_plain / steps_plain,
                       "mixed_over_plain": value / value_plain},
        "rmse": out_rmse,
        "e2e": {"value": e2e_value, "unit": "Mphotons/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "step": f"ppm_scene_upload + ppm_camera_set + ppm_render({w['passes']} passes, cell size {cells} "
                        f"as tuned above) + image download"},
        "gpu_launches": kernels_per_pass * args.steps,
        "kernels_per_pass": kernels_per_pass,
        "stages_ms_per_pass": {k: round(v, 4) for k, v in stage_avg.items()},
        "roofline": {"kernel": dominant, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                     "algorithmic_bytes": ab},
        "stage_rooflines": stage_roof,
        "rates": rates,
        "pass_stats": {"photons_stored": st["photons_stored"], "hit_points": st["hit_points"],
                       "grid_cells": st["grid_cells"]},
        "cpu_baseline": cpu,
        "clocks": clk,
    }
    print(json.dumps(out))


def hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        return json.load(open(path))["hbm_gbs"], "measured"
    return 6800.0, "fallback"


def sweep_inputs(args, kind):
    from ppmpa_gb300 import workloads as W
    pos, d, wl = W.photons(args.sweep_photons, kind)
    q, nrm, r2 = W.queries(args.sweep_queries, kind)
    return pos, d, wl, q, nrm, r2


def run_sweep(args, kind):
    """One step = one ppm_estimate_f32 call over all queries (host arrays in,
    host results out).  value: estimates per second of the device work (query
    sort + gather); e2e: the same through the call with its copies."""
    import torch
    from ppmpa_gb300 import Context, workloads as W
    t0 = time.perf_counter()
    pos, d, wl, q, nrm, r2 = sweep_inputs(args, kind)
    gen_s = time.perf_counter() - t0
    n_ph, n_q = len(pos), len(q)
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
    for _ in range(max(3, args.warmup)):
        ctx.estimate_f32(q, nrm, r2)
    base = ctx.stats()
    clocks = Clocks(0)
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.estimate_f32(q, nrm, r2)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    st = ctx.stats()
    ctx.close()
    gather_ms = (st["stage_ms"]["gather"] - base["stage_ms"]["gather"]) / args.steps
    sort_ms = (st["stage_ms"]["query_sort"] - base["stage_ms"]["query_sort"]) / args.steps
    dev_ms = gather_ms + sort_ms
    peak, src = hbm_peak()
    photon_bytes = 16                               # float3 position + packed direction/wavelength
    query_bytes = 12 + 12 + 8 + 24                  # position, normal, radius^2 in; RGB out
    ab = n_ph * photon_bytes + n_q * query_bytes
    achieved = ab / (gather_ms / 1e3) / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(prof):
        traffic = json.load(open(prof)).get(args.workload)
    out = {
        "metric": f"gather sweep estimates/s ({n_ph} FP32 photons, {n_q} queries, r log-uniform 1e-3..2e-2)",
        "value": n_q / (dev_ms / 1e3) / 1e6, "unit": "Mqueries/s", "n_gpus": 1, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": dev_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 positions/tests, f64 rounding-band recheck and normalisation",
        "data": "synthetic (seeded photons and queries)",
        "config": {"workload": args.workload, "distribution": kind, "photons": n_ph, "queries": n_q,
                   "r_min": W.R_MIN, "r_max": W.R_MAX, "cells_per_radius": cells, "autotune": tune,
                   "l2": f"inputs larger than L2 (map {n_ph * photon_bytes / 2**30:.2f} GiB)"},
        "gather_ms": gather_ms, "query_sort_ms": sort_ms, "map_build_ms": build_ms,
        "photon_tests_per_s": cnt["candidates"] / (gather_ms / 1e3), "in_radius_per_s": cnt["in_radius"] / (gather_ms / 1e3),
        "candidates": cnt["candidates"], "in_radius": cnt["in_radius"], "lane_slots": cnt["gather_slots"],
        "e2e": {"value": n_q * args.steps / wall / 1e6, "unit": "Mqueries/s",
                "h2d_bytes_per_step": n_q * (12 + 12 + 8), "d2h_bytes_per_step": n_q * 24,
                "step": "ppm_estimate_f32 over all queries, pageable host arrays"},
        "gpu_launches": 6 * args.steps,
        "roofline": {"kernel": "gather", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": src, "algorithmic_bytes": ab},
        "input_generation_s": gen_s, "clocks": clk,
    }
    print(json.dumps(out), flush=True)


def run_sweep_reference(args, kind):
    """The FP64 restatement of the reference's estimate (grid in place of the
    kd-tree) over the same map, on a bounded sample of the queries."""
    from oracle.binding import Oracle
    from ppmpa_gb300 import scene as S
    pos, d, wl, q, nrm, r2 = sweep_inputs(args, kind)
    orc = Oracle(S.Scene(), threads=0)
    threads = orc.L.orc_get_threads()
    p64, d64 = pos.astype(np.float64), d.astype(np.float64)
    n_s = min(len(q), 20000)
    qs, ns, rs = q[:n_s].astype(np.float64), nrm[:n_s].astype(np.float64), r2[:n_s]
    total = 0.0
    for k in range(max(1, args.warmup) + args.steps):
        orc.estimate_radii(p64, d64, wl, qs, ns, rs, 1.0 / len(pos))
        if k >= max(1, args.warmup):
            total += orc.L.orc_last_query_seconds()   # query phase; the grid build is not timed
    value = n_s * args.steps / total / 1e6
    sample = f"{n_s} of the queries per step over the full map, {threads} threads, grid build excluded"
    print(json.dumps({
        "impl": "reference", "metric": f"gather sweep estimates/s ({len(pos)} FP32 photons, {len(q)} queries, "
                                       f"r log-uniform 1e-3..2e-2)",
        "value": value, "unit": "Mqueries/s", "n_gpus": args.gpus, "host_only": True, "steps": args.steps,
        "warmup": max(1, args.warmup),
        "ms_per_step": total / args.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded photons and queries)",
        "config": {"workload": args.workload, "distribution": kind, "photons": len(pos), "queries": len(q)},
        "cpu_baseline": {"value": value, "unit": "Mqueries/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "Mqueries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def run_batch(args, bw):
    """A step = one pass of every job.  value: photons of all jobs per second
    of batch device time; sequential: the same jobs rendered one after
    another, each with its own pass graph; e2e: Batch.render wall time
    (scene uploads, BVH builds, cell tuning, graph capture, passes, images)."""
    import torch
    from ppmpa_gb300 import Batch, Context, workloads as W
    jobs = W.batch_jobs(bw["n_jobs"], seed=args.seed + 6, passes=bw["passes"])
    photons = sum(cfg.nphoton for _, _, cfg in jobs) * bw["passes"]
    with Batch(0, seed=args.seed) as b:
        b.render(jobs)                                   # warm-up: allocations, module loads
        clocks = Clocks(0)
        clocks.start()
        t0 = time.perf_counter()
        imgs, dev_ms = b.render(jobs)
        wall = time.perf_counter() - t0
        clk = clocks.stop()
    seq_ms = 0.0
    with Context(0, seed=args.seed) as ctx:
        for sc, cam, cfg in jobs:
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
    out = {
        "metric": f"batched render Mphotons/s ({len(jobs)} uneven jobs, one graph launch per pass)",
        "value": photons / (dev_ms / 1e3) / 1e6, "unit": "Mphotons/s", "n_gpus": 1, "steps": bw["passes"],
        "warmup": 1, "ms_per_step": dev_ms / bw["passes"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 trace/gather, f64 radius/average", "data": "synthetic (seeded scenes)",
        "config": {"workload": args.workload, "jobs": len(jobs), "passes": bw["passes"],
                   "primitives": [min(prims), max(prims), sum(prims)],
                   "photons_per_pass": [min(c.nphoton for _, _, c in jobs), max(c.nphoton for _, _, c in jobs)],
                   "reso": [min(c.xreso for _, c, _ in jobs), max(c.xreso for _, c, _ in jobs)],
                   "cell_tuning": True},
        "sequential": {"value": photons / (seq_ms / 1e3) / 1e6, "unit": "Mphotons/s", "ms": seq_ms},
        "batch_over_sequential": seq_ms / dev_ms,
        "e2e": {"value": photons / wall / 1e6, "unit": "Mphotons/s",
                "h2d_bytes_per_step": sum(120 * sc.n_objects + 168 * len(sc.materials) + 160 * len(sc.lights) + 336
                                          for sc, _, _ in jobs),
                "d2h_bytes_per_step": sum(i.nbytes for i in imgs),
                "step": "Batch.render: uploads, BVH builds, tuning, capture, all passes, images"},
        "mean_radiance": float(np.mean([i.mean() for i in imgs])), "clocks": clk,
    }
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.workload in BATCHES:
        if dist_env()[0] == 0 and args.impl != "reference":
            run_batch(args, BATCHES[args.workload])
        elif dist_env()[0] == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the batch workload has no CPU leg: the reference "
                              "tests every object per ray and renders one scene per process"}))
        return
    if args.nphoton > 0 and args.workload in WORKLOADS:
        WORKLOADS[args.workload] = dict(WORKLOADS[args.workload], nphoton=args.nphoton)
    if args.workload in SWEEPS:
        rank, world, _ = dist_env()
        if rank == 0:
            (run_sweep_reference if args.impl == "reference" else run_sweep)(args, SWEEPS[args.workload])
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

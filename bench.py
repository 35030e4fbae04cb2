#!/usr/bin/env python3
"""Benchmark of the path-tracing hot path on the 1920x1080 production scene.

Workload: bonsai_gb300.scenes.production() - 64 fBm-displaced level-5 icospheres (1.31M triangles),
2000 lognormal spheres, ground quad, 4 quad area lights; 1920x1080, 64 spp, max depth 8, Russian
roulette after depth 3, PBRT estimator (unbiased), seeded synthetic geometry.

One step = one full 64-spp render of the frame (132.7M samples).
  value : Msamples/s on the device: samples / sum of CUDA-event render times (scene resident in
          HBM, film left on the device), L2 flushed (512 MB write) before every step.
  e2e   : Msamples/s through the C ABI entry point bg_render with a host film buffer: every step
          sends the camera/options and reads the resolved 1920x1080x3 float film back.
  roofline: dominant kernel = closest-hit traversal (k_extend).  Algorithmic bytes per ray =
          32 (ray) + 8 (hit) + 32 V + 40 T, with V / T the mean node visits / triangle tests of the
          reference traversal (binary SAH BVH, bucket-fixed build) counted by the CPU oracle on a
          subsample of the same paths; achieved = bytes / summed k_extend event time.
  cpu_baseline: the CPU oracle (C++ restatement of the reference, PBRT mode, bucket-fixed BVH) on
          all host cores over a bounded subset of image rows.
--impl reference times that same CPU restatement as the reference arm.
Multi-GPU (--gpus N under torchrun): independent replicas, one per GPU ("replicas only").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Msamples/s"
UNIT = "Msamples/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--small", action="store_true", help="reduced scene for quick checks (not a bench line)")
    p.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU work of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--profile", action="store_true",
                   help="profiling case for ncu: one render of the full-size scene at --profile-spp spp")
    p.add_argument("--profile-spp", type=int, default=1)
    p.add_argument("--no-autotune", action="store_true")
    p.add_argument("--workload", choices=["production", "raysoup", "guiding", "guide-mlp", "batch", "whitted", "direct",
                                          "example", "relmse", "guided-pass"],
                   default="production",
                   help="raysoup: the 2M-triangle / 16M-ray closest-hit + any-hit microbenchmark (Mrays/s); "
                        "guiding: time-to-relMSE 1e-3 of guided vs plain path tracing on the slit room; "
                        "example: the reference's example scene (UV-textured sphere under an environment map); "
                        "relmse: relMSE of the Cornell (256^2, 16 spp) and 1080p (64 spp) renders against "
                        "--ref-spp renders of the same scene and mode; "
                        "guided-pass: device time of one 4-spp slit room pass, plain, guided with a frozen network "
                        "and guided with training (with --profile: a profiler window around the last repetition)")
    p.add_argument("--ref-spp", type=int, default=16384, help="guiding: spp of the plain reference render")
    p.add_argument("--arm-seconds", type=float, default=90.0, help="guiding: time limit of each progressive arm")
    p.add_argument("--target", type=float, default=1e-3, help="guiding: relMSE target")
    p.add_argument("--guide-warmup", type=int, default=8, help="guiding: unguided training passes")
    p.add_argument("--pass-paths", type=int, default=1 << 22, help="guiding: paths per pass")
    p.add_argument("--epochs", type=int, default=2, help="guiding: training epochs over each pass's pool")
    p.add_argument("--pool", type=int, default=1 << 18, help="guiding: training samples gathered per pass")
    p.add_argument("--guided-scenes", type=int, default=8, help="batch: scenes of the guided arm (0 = none)")
    p.add_argument("--guided-train-passes", type=int, default=64, help="batch: training passes per guided scene")
    return p.parse_args()


def workload(small: bool):
    from bonsai_gb300 import scenes as S
    if small:
        return S.production(480, 270, spp=16, max_depth=8, n_ico=8, ico_level=4, n_spheres=500)
    return S.production()


def config_of(sd, small: bool) -> dict:
    return {
        "workload": ("production-small" if small else "production 1080p") +
                    f": {sd.ntri} triangles ({sd.meta.get('n_ico', 64)} fBm icospheres "
                    f"L{sd.meta.get('ico_level', 5)} + ground + 4 quad lights), "
                    f"{sd.nsph} spheres, {sd.camera.width}x{sd.camera.height}, {sd.spp} spp, max depth "
                    f"{sd.max_depth}, RR after depth 3, PBRT estimator",
        "width": sd.camera.width, "height": sd.camera.height, "spp": sd.spp, "max_depth": sd.max_depth,
        "triangles": sd.ntri, "spheres": sd.nsph, "bvh": "8-wide compressed (80 B nodes, 8-bit child boxes, <= 2 primitives per leaf)", "graph": "wave chain captured as a CUDA graph",
        "l2": "flushed before every step (512 MB device write)",
        "parallelism": "replicas",
    }


def example_config(sd, small: bool) -> dict:
    e = sd.env.rgb.shape
    return {
        "workload": f"reference example scene (src/main.rs){' small' if small else ''}: unit sphere, matte with a "
                    f"UVTexture, InfiniteAreaLight with a {e[1]}x{e[0]} synthetic environment map, "
                    f"{sd.camera.width}x{sd.camera.height}, {sd.spp} spp, max depth {sd.max_depth}, "
                    f"RR threshold {sd.rr_threshold}, PBRT estimator",
        "width": sd.camera.width, "height": sd.camera.height, "spp": sd.spp, "max_depth": sd.max_depth,
        "integrator": "PathIntegrator", "env_map": [int(e[1]), int(e[0])],
        "sampler": "StratifiedSampler 4x4, 4 sampled dimensions, jitter",
        "bvh": "8-wide compressed", "graph": "wave chain captured as a CUDA graph",
        "l2": "flushed before every step (512 MB device write)", "parallelism": "replicas",
    }


# ---------------------------------------------------------------- distributed (replicas only)
def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0, None
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist.get_rank(), ws, int(os.environ.get("LOCAL_RANK", "0")), dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- clocks
class Clocks:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        loaded = [s for s in sm if s > 0.5 * (max(mx) if mx else 0)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------- CPU baseline (oracle)
def cpu_sample(sd, target_s: float, threads: int, **kw):
    """Times the CPU restatement over every k-th image row, k chosen for ~target_s of work."""
    import oracle as O
    from bonsai_gb300 import _abi as A
    t0 = time.time()
    orc = O.OracleScene(sd, fixed_bvh=True)
    build_s = time.time() - t0
    H, W = sd.camera.height, sd.camera.width
    probe_rows = (0, H, max(1, H // 8))
    t0 = time.time()
    probe_spp = sd.spp if kw.get("sampler") is not None else max(1, sd.spp // 16)  # a stratified pass is whole
    orc.render(A.BG_MODE_PBRT, spp=probe_spp, rows=probe_rows, threads=threads, **kw)
    dt = max(time.time() - t0, 1e-3)
    probe_samples = len(range(*probe_rows)) * W * probe_spp
    rate = probe_samples / dt
    want_rows = max(1, int(target_s * rate / (W * sd.spp)))
    step = max(1, H // want_rows)
    rows = (0, H, step)
    nrows = len(range(*rows))
    return orc, rows, nrows * W * sd.spp, build_s


def time_cpu(orc, sd, rows, nsamples, threads, **kw):
    from bonsai_gb300 import _abi as A
    t0 = time.time()
    orc.render(A.BG_MODE_PBRT, rows=rows, threads=threads, **kw)
    dt = time.time() - t0
    return nsamples / dt / 1e6, dt


def traversal_counts(orc, sd):
    """Mean node visits / primitive tests per closest-hit and any-hit ray of the reference
    traversal, on the paths of a row subsample (1 spp)."""
    from bonsai_gb300 import _abi as A
    H = sd.camera.height
    r = orc.render(A.BG_MODE_PBRT, spp=2, rows=(0, H, max(1, H // 24)), count_traversal=True)
    c = r["counters"]
    return {"V_ext": c[2] / max(c[0], 1), "T_ext": c[3] / max(c[0], 1),
            "V_sh": c[4] / max(c[1], 1), "T_sh": c[5] / max(c[1], 1), "rays_counted": int(c[0] + c[1])}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------- arms
def run_reference(args):
    rank, ws, local, dist = dist_init()
    if rank != 0:
        return
    sd = workload(args.small)
    threads = os.cpu_count() or 1
    orc, rows, nsamples, build_s = cpu_sample(sd, min(args.cpu_seconds, 20.0), threads)
    for _ in range(args.warmup):
        time_cpu(orc, sd, rows, nsamples, threads)
    vals, times = [], []
    for _ in range(args.steps):
        v, dt = time_cpu(orc, sd, rows, nsamples, threads)
        vals.append(v)
        times.append(dt)
    total_t = sum(times)
    value = args.steps * nsamples / total_t / 1e6
    sample = (f"rows 0..{sd.camera.height} step {rows[2]} ({len(range(*rows))} rows x {sd.camera.width} px x "
              f"{sd.spp} spp = {nsamples} samples per step)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total_t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": config_of(sd, args.small),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "notes": "C++ restatement of the reference PathIntegrator (oracle/), PBRT estimator, bucket-fixed "
                 "reference BVH (the reference's own bucket bug makes a chain BVH); the Rust reference cannot "
                 f"be built here (no Rust toolchain). Oracle BVH build {build_s:.1f} s excluded.",
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    from bonsai_gb300 import _abi as A
    from bonsai_gb300 import gpu as G
    rank, ws, local, dist = dist_init()
    sd = workload(args.small)
    ctx = G.Context(local)
    t0 = time.time()
    scene = G.Scene(ctx, sd, A.BG_BVH_WIDE)
    upload_build_s = time.time() - t0
    pi = G.PathIntegrator(sd.camera, sd.spp, sd.max_depth, sd.rr_threshold, mode=A.BG_MODE_PBRT, seed=0)
    samples = sd.camera.width * sd.camera.height * sd.spp
    tuning = None
    if not args.no_autotune:
        from bonsai_gb300 import autotune
        tuning = autotune.tune(ctx, scene, pi, spp=4)
        tuning = {k: tuning[k] for k in ("refill", "blocks_per_sm", "wave_paths", "sort_rays", "concurrent_shade", "ms")} | {
            "cached": bool(tuning.get("cached", False))}
        # traversal node width: the scene rebuilt 8-wide and 2-wide, the faster kept
        scene.close()
        scene, lay = autotune.tune_layout(ctx, sd, pi, spp=4)
        tuning["node_width"] = 8 if lay["layout"] == A.BG_BVH_WIDE else 2
        tuning["node_width_trials_ms"] = {("8" if t["layout"] == A.BG_BVH_WIDE else "2"): t["ms"]
                                          for t in lay.get("trials", [])}
    for _ in range(args.warmup):
        pi.render(scene, readback=False, graph=True)
    clocks = Clocks(local)
    barrier(dist)
    ctx.synchronize()
    clocks.start()
    dev_ms, launches, wall0 = 0.0, 0, time.time()
    for k in range(args.steps):
        ctx.flush_l2()
        r = pi.render(scene, readback=False, first_sample=k * sd.spp, graph=True)
        dev_ms += r.stats.device_ms
        launches += r.stats.launches
        if r.stats.error_word:
            raise RuntimeError(f"device error word {r.stats.error_word}")
    ctx.synchronize()
    wall = time.time() - wall0
    clk = clocks.stop()
    barrier(dist)
    dev_ms_max = max_over_ranks(dist, dev_ms)
    value = ws * args.steps * samples / (dev_ms_max / 1e3) / 1e6

    # end to end through the C ABI with a host film buffer (read back every step)
    barrier(dist)
    t0 = time.time()
    for k in range(args.steps):
        pi.render(scene, readback=True, first_sample=k * sd.spp, graph=True)
    e2e_s = max_over_ranks(dist, time.time() - t0)

    # the plain wavefront arm (kernel launches, no graph) at the same tuning, one timed frame
    ctx.flush_l2()
    plain = pi.render(scene, readback=False)
    plain_msps = samples / (plain.stats.device_ms / 1e3) / 1e6
    e2e = ws * args.steps * samples / e2e_s / 1e6

    # stage timing pass (outside the timed region): dominant-kernel duration and ray counts
    o = A.bg_render_opts()
    ctx.flush_l2()
    import ctypes as C
    cam = G.camera_struct(sd.camera)
    o.spp, o.max_depth, o.rr_threshold, o.mode, o.seed = sd.spp, sd.max_depth, sd.rr_threshold, A.BG_MODE_PBRT, 0
    o.flags = A.BG_RENDER_NO_READBACK | A.BG_RENDER_STAGE_TIMING
    st = A.bg_render_stats()
    ctx.check(ctx.lib.bg_render(ctx.h, scene.h, C.byref(cam), C.byref(o), None, C.byref(st)))
    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    roof = {"bound": "hbm", "achieved": None, "peak": peak, "unit": "GB/s", "frac": None, "traffic": None,
            "kernel": "k_extend<8> (closest hit, 8-wide compressed BVH)", "peak_source": peak_kind}
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        orc, rows, nsamples, build_s = cpu_sample(sd, args.cpu_seconds, threads)
        counts = traversal_counts(orc, sd)
        bpr = 32 + 8 + 32 * counts["V_ext"] + 40 * counts["T_ext"]
        achieved = st.extension_rays * bpr / (st.trace_ms / 1e3) / 1e9
        roof.update({"achieved": achieved, "frac": achieved / peak, "bytes_per_ray": bpr, **counts})
        tp = ROOT / "profiles" / "k_extend_traffic.json"
        if tp.exists():  # DRAM bytes of one captured launch (ncu), per ray, against the algorithmic bytes
            t = json.loads(tp.read_text())
            roof["traffic"] = t["dram_bytes_read"] + t["dram_bytes_write"]
            roof["traffic_launch"] = {"rays": t["rays"], "algorithmic_bytes": t["rays"] * bpr,
                                      "dram_bytes_per_ray": roof["traffic"] / t["rays"], "workload": t["workload"]}
        cv, cdt = time_cpu(orc, sd, rows, nsamples, threads)
        cpu = {"value": cv, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"rows 0..{sd.camera.height} step {rows[2]} x {sd.camera.width} px x {sd.spp} spp "
                         f"= {nsamples} samples in {cdt:.1f} s (oracle/, PBRT mode, bucket-fixed BVH)"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded scene generator, bonsai_gb300/scenes.py)",
        "config": config_of(sd, args.small) | {"tuning": tuning} | (
            {"bvh": "2-wide (64 B nodes; the autotuner's node-width choice)"}
            if tuning and tuning.get("node_width") == 2 else {}),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": C.sizeof(A.bg_camera) + C.sizeof(A.bg_render_opts),
                "d2h_bytes_per_step": sd.camera.width * sd.camera.height * 3 * 4},
        "gpu_launches": launches,
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clk,
        "extra": {"plain_wavefront_msamples_per_s": plain_msps, "wall_s_timed_loop": wall, "scene_upload_and_bvh_build_s": upload_build_s,
                  "bvh_build_ms": scene.build_ms, "bvh_nodes": int(scene.nodes),
                  "extension_rays_per_frame": int(st.extension_rays), "shadow_rays_per_frame": int(st.shadow_rays),
                  "Mrays_per_s": (st.extension_rays + st.shadow_rays) / (st.device_ms / 1e3) / 1e6,
                  "stage_ms": {"extend": st.trace_ms, "shade": st.shade_ms, "shadow": st.shadow_ms,
                               "total": st.device_ms}},
    }
    print(json.dumps(line), flush=True)


def example_workload(small: bool):
    """The reference's example program (src/main.rs): a unit sphere, matte with a UVTexture, under an
    InfiniteAreaLight of identity transform, 1024x1024, 16 spp (its 4x4 stratified sampler), path
    depth 5, roulette threshold 1; the environment map is a seeded synthetic 2048x1024 sky."""
    from bonsai_gb300 import scenes as S
    if small:
        return S.env_sphere(256, 256, spp=16, max_depth=5, env_w=512, env_h=256)
    return S.env_sphere(1024, 1024, spp=16, max_depth=5, env_w=2048, env_h=1024)


def run_integrators(args):
    """The Whitted (`--workload whitted`) and direct-lighting (`--workload direct`, UniformSampleAll:
    every light with MIS) integrators on the production scene, or the path integrator on the
    reference's example scene (`--workload example`): value = device Msamples/s over K frames (L2
    flushed), e2e through bg_render with the film read back; CPU restatement of the same
    integrator (oracle/) on all host cores.  The ray trees run as a breadth-first wavefront over
    the 8-wide BVH (bonsai_gb300/csrc/bg_tree_wave.cu)."""
    import ctypes as C
    from bonsai_gb300 import _abi as A
    from bonsai_gb300 import gpu as G
    rank, ws, local, dist = dist_init()
    sd = example_workload(args.small) if args.workload == "example" else workload(args.small)
    graph = False
    extra_kw = {}
    if args.workload == "example":
        from bonsai_gb300 import scenes as S
        kind, strategy, name = A.BG_INTEGRATOR_PATH, 0, "PathIntegrator"
        smp = S.StratifiedSampler(4, 4, 4, True)  # src/main.rs: StratifiedSampler 4 x 4, 4 dimensions, jitter
        integ = lambda: G.PathIntegrator(sd.camera, sd.spp, sd.max_depth, sd.rr_threshold,  # noqa: E731
                                         mode=A.BG_MODE_PBRT, sampler=smp)
        extra_kw = {"sampler": smp}
        graph = True
    elif args.workload == "whitted":
        kind, strategy, name = A.BG_INTEGRATOR_WHITTED, 0, "WhittedIntegrator"
        integ = lambda: G.WhittedIntegrator(sd.camera, sd.spp, sd.max_depth, mode=A.BG_MODE_PBRT)  # noqa: E731
    else:
        kind, strategy, name = A.BG_INTEGRATOR_DIRECT, A.BG_LIGHT_UNIFORM_ALL, "DirectLightingIntegrator(UniformSampleAll)"
        integ = lambda: G.DirectLightingIntegrator(sd.camera, sd.spp, sd.max_depth, strategy,  # noqa: E731
                                                   mode=A.BG_MODE_PBRT)
    ctx = G.Context(local)
    scene = G.Scene(ctx, sd, A.BG_BVH_WIDE)
    pi = integ()
    samples = sd.camera.width * sd.camera.height * sd.spp
    gkw = {"graph": True} if graph else {}
    for _ in range(args.warmup):
        pi.render(scene, readback=False, **gkw)
    clocks = Clocks(local)
    barrier(dist)
    ctx.synchronize()
    clocks.start()
    dev_ms, launches, rays = 0.0, 0, 0
    for k in range(args.steps):
        ctx.flush_l2()
        r = pi.render(scene, readback=False, first_sample=k * sd.spp, **gkw)
        dev_ms += r.stats.device_ms
        launches += r.stats.launches
        rays += r.stats.extension_rays + r.stats.shadow_rays
        if r.stats.error_word:
            raise RuntimeError(f"device error word {r.stats.error_word}")
    ctx.synchronize()
    clk = clocks.stop()
    barrier(dist)
    dev_ms_max = max_over_ranks(dist, dev_ms)
    value = ws * args.steps * samples / (dev_ms_max / 1e3) / 1e6
    barrier(dist)
    t0 = time.time()
    for k in range(args.steps):
        pi.render(scene, readback=True, first_sample=k * sd.spp, **gkw)
    e2e = ws * args.steps * samples / max_over_ranks(dist, time.time() - t0) / 1e6
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        kw = {"integrator": kind, "light_strategy": strategy} | extra_kw
        orc, rows, nsamples, _ = cpu_sample(sd, args.cpu_seconds, threads, **kw)
        cv, cdt = time_cpu(orc, sd, rows, nsamples, threads, **kw)
        cpu = {"value": cv, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"rows 0..{sd.camera.height} step {rows[2]} x {sd.camera.width} px x {sd.spp} spp "
                         f"= {nsamples} samples in {cdt:.1f} s (oracle/, PBRT mode, bucket-fixed BVH)"}
    peak, peak_kind = measured_peaks()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded scene generator, bonsai_gb300/scenes.py)",
        "config": (example_config(sd, args.small) if args.workload == "example" else
                   config_of(sd, args.small) | {"integrator": name, "graph": "no (a host check per wave)",
                                                "waves": "breadth-first ray-tree wavefront, <= 2M samples per wave"}),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": C.sizeof(A.bg_camera) + C.sizeof(A.bg_render_opts),
                "d2h_bytes_per_step": sd.camera.width * sd.camera.height * 3 * 4},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": None, "peak": peak, "unit": "GB/s", "frac": None, "traffic": None,
                     "kernel": ("k_extend<8> / k_shadow<8> (path wavefront)" if graph else
                                "k_tw_extend<8> / k_tw_shadow<8> (tree wavefront)"), "peak_source": peak_kind,
                     "note": "the traversal kernels are those of the production path workload, which carries "
                             "the roofline"},
        "cpu_baseline": cpu,
        "clocks": clk,
        "extra": {"rays_per_frame": rays // args.steps, "Mrays_per_s": rays / (dev_ms / 1e3) / 1e6},
    }
    print(json.dumps(line), flush=True)


def run_profile(args):
    """One render of the production scene (full geometry and resolution, few spp): the case the ncu
    launch list and kernel captures run on (a few GB on the device, BVH larger than L2)."""
    from bonsai_gb300 import _abi as A
    from bonsai_gb300 import gpu as G
    from bonsai_gb300 import autotune
    sd = workload(False)
    ctx = G.Context(0)
    scene = G.Scene(ctx, sd, A.BG_BVH_WIDE)
    # the launch shape the autotuner picks for the production bench on a GB300 (refill 8, 16 CTAs
    # per SM, 16M-path waves)
    autotune.set_(ctx, 8, 16, 1 << 24)
    pi = G.PathIntegrator(sd.camera, args.profile_spp, sd.max_depth, sd.rr_threshold, mode=A.BG_MODE_PBRT)
    r = pi.render(scene, readback=False)
    print(json.dumps({"profile_case": True, "spp": args.profile_spp, "device_ms": r.stats.device_ms,
                      "launches": int(r.stats.launches), "extension_rays": int(r.stats.extension_rays),
                      "shadow_rays": int(r.stats.shadow_rays)}))
    scene.close()
    ctx.close()


def run_raysoup(args):
    """Ray/BVH microbenchmark: 2,097,152 random triangles (seed 1), 16,777,216 random rays (seed 2),
    closest-hit and any-hit queries.  value = (closest + any) rays / summed kernel time, rays and
    results resident on the device; e2e = the same through bg_trace_closest / bg_trace_any with host
    arrays (copies included)."""
    import ctypes as C
    from bonsai_gb300 import _abi as A
    from bonsai_gb300 import gpu as G
    from bonsai_gb300 import scenes as S
    ntri, nrays = (262_144, 2_097_152) if args.small else (2_097_152, 16_777_216)
    sd, rays = S.ray_soup(ntri, nrays)
    ctx = G.Context(0)
    t0 = time.time()
    scene = G.Scene(ctx, sd, A.BG_BVH_WIDE)
    build_s = time.time() - t0
    d_rays = ctx.alloc(rays.nbytes)
    d_hits = ctx.alloc(nrays * 8)
    d_occ = ctx.alloc(nrays)
    ctx.h2d(d_rays, rays)
    for _ in range(args.warmup):
        scene.trace_device(d_rays, nrays, d_hits)
        scene.trace_device(d_rays, nrays, d_occ, any_hit=True)
    clocks = Clocks(0)
    clocks.start()
    ms_c = ms_a = 0.0
    for _ in range(args.steps):
        ctx.flush_l2()
        ms_c += scene.trace_device(d_rays, nrays, d_hits)
        ctx.flush_l2()
        ms_a += scene.trace_device(d_rays, nrays, d_occ, any_hit=True)
    clk = clocks.stop()
    value = 2 * nrays * args.steps / ((ms_c + ms_a) / 1e3) / 1e6
    t0 = time.time()
    for _ in range(args.steps):
        hits = scene.trace(rays)
        occ = scene.trace(rays, any_hit=True)
    e2e = 2 * nrays * args.steps / (time.time() - t0) / 1e6
    consistent = bool(np.array_equal(occ.astype(bool), hits["prim"] >= 0))
    roof, cpu = None, None
    peak, peak_kind = measured_peaks()
    if not args.no_cpu_baseline:
        import oracle as O
        threads = os.cpu_count() or 1
        orc = O.OracleScene(sd, fixed_bvh=True)
        sub = rays[:: max(1, nrays // 200_000)]
        hc, cc = orc.trace(sub, count=True, threads=threads)
        ha, ca = orc.trace(sub, any_hit=True, count=True, threads=threads)
        V_c, T_c = cc[0] / len(sub), cc[1] / len(sub)
        V_a, T_a = ca[0] / len(sub), ca[1] / len(sub)
        bytes_c = 32 + 8 + 32 * V_c + 40 * T_c
        bytes_a = 32 + 1 + 32 * V_a + 40 * T_a
        achieved = nrays * args.steps * bytes_c / (ms_c / 1e3) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": None, "kernel": "k_trace<8,closest> (8-wide BVH)", "peak_source": peak_kind,
                "bytes_per_ray_closest": bytes_c, "bytes_per_ray_any": bytes_a, "V_closest": V_c, "T_closest": T_c,
                "V_any": V_a, "T_any": T_a}
        mism = int((hc["prim"] != hits["prim"][:: max(1, nrays // 200_000)][:len(sub)]).sum())
        t0 = time.time()
        orc.trace(rays[: 4 * len(sub)], threads=threads)
        orc.trace(rays[: 4 * len(sub)], any_hit=True, threads=threads)
        cdt = time.time() - t0
        cpu = {"value": 2 * 4 * len(sub) / cdt / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
               "sample": f"first {4 * len(sub)} rays, closest + any (oracle/, bucket-fixed reference BVH)",
               "subsample_prim_mismatches": mism, "subsample_rays": len(sub)}
    print(json.dumps({
        "metric": "Mrays/s (closest + any)", "value": value, "unit": "Mrays/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": (ms_c + ms_a) / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": f"ray soup: {ntri} random triangles (seed 1), {nrays} random rays (seed 2)",
                   "bvh": "8-wide compressed", "l2": "flushed before every query"},
        "e2e": {"value": e2e, "unit": "Mrays/s", "h2d_bytes_per_step": 2 * rays.nbytes,
                "d2h_bytes_per_step": nrays * 8 + nrays},
        "closest_mrays": nrays * args.steps / (ms_c / 1e3) / 1e6, "any_mrays": nrays * args.steps / (ms_a / 1e3) / 1e6,
        "any_consistent_with_closest": consistent, "bvh_build_s": build_s, "roofline": roof, "cpu_baseline": cpu,
        "clocks": clk}), flush=True)
    scene.close()
    ctx.close()


def _relmse(img, ref, ref_var_term):
    """mean over pixels and channels of (x - ref)^2 / (ref^2 + 0.01), minus the reference's own
    expected contribution (its per-pixel variance of the mean over the same denominator)."""
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)) - ref_var_term)


def _time_to(curve, target):
    """First crossing of `target` by log-log interpolation between checkpoints; if the curve never
    reaches it, extrapolation from the last checkpoint with relMSE ~ 1/t.  Returns (t, extrapolated)."""
    if curve and curve[0][1] <= target:
        return curve[0][0], False
    for (t0, e0), (t1, e1) in zip(curve, curve[1:]):
        if e0 > target >= e1 and e0 > 0 and e1 > 0:
            a = (np.log(target) - np.log(e0)) / (np.log(e1) - np.log(e0))
            return float(np.exp(np.log(t0) + a * (np.log(t1) - np.log(t0)))), False
    t, e = curve[-1]
    return float(t * max(e, 0.0) / target), True


def _at_time(curve, t):
    """relMSE at time t (log-log interpolation inside the curve)."""
    for (t0, e0), (t1, e1) in zip(curve, curve[1:]):
        if t0 <= t <= t1 and e0 > 0 and e1 > 0:
            a = (np.log(t) - np.log(t0)) / (np.log(t1) - np.log(t0))
            return float(np.exp(np.log(e0) + a * (np.log(e1) - np.log(e0))))
    return None


def run_guiding(args):
    """Learned path guiding on the slit room (1280x720, max depth 10, 204,816 triangles, 200
    spheres): time-to-relMSE 1e-3 of the guided progressive render (online training included in
    the timed region) against plain graph-captured path tracing, both measured against a plain
    reference render, plus relMSE at equal time.  The CPU number is derived: the oracle runs the
    same estimator as the plain GPU arm, so its time to the target is the plain arm's samples to the
    target divided by the oracle's measured Msamples/s on this scene."""
    from bonsai_gb300 import _abi as A
    from bonsai_gb300 import gpu as G
    from bonsai_gb300 import scenes as S
    if args.small:
        sd = S.slit_room(320, 180, n_ico=10, ico_level=3, n_spheres=200, light_intensity=200.0)
    else:
        sd = S.slit_room(light_intensity=200.0)
    W, H = sd.camera.width, sd.camera.height
    npix = W * H
    ctx = G.Context(0)
    scene = G.Scene(ctx, sd, A.BG_BVH_WIDE)
    pi = G.PathIntegrator(sd.camera, 1, sd.max_depth, sd.rr_threshold, mode=A.BG_MODE_PBRT, seed=11)

    def mean_image():
        s1, s2, n = G.PathIntegrator.moments(ctx, W, H)
        n = np.maximum(n[..., None], 1).astype(np.float64)
        return s1 / n, s2 / n, n

    # reference: plain, ref_spp, separate sample indices
    t0 = time.time()
    chunk = 256
    for k in range(0, args.ref_spp, chunk):
        pi.render(scene, spp=min(chunk, args.ref_spp - k), first_sample=(1 << 26) + k, accumulate=k > 0,
                  readback=False, graph=True)
    ref, ref2, refn = mean_image()
    ref_var_term = float(np.mean(np.maximum(ref2 - ref * ref, 0.0) / refn / (ref ** 2 + 1e-2)))
    ref_s = time.time() - t0

    moments_est = {}

    def progressive(render_chunk, label):
        curve, t_dev, t_wall, spp, c = [], 0.0, 0.0, 0, 4
        while True:
            w0 = time.time()
            st = render_chunk(c, spp)
            t_wall += time.time() - w0
            t_dev += st.device_ms / 1e3
            spp += c
            img, img2, n = mean_image()
            e = _relmse(img, ref, ref_var_term)
            curve.append((t_dev, e, t_wall, spp))
            if e < args.target / 1.5 or t_dev > args.arm_seconds:
                break
            c = max(4, int(c * 1.3))
        # the arm's own estimate of its relMSE (per-pixel sample variance of the mean, no reference),
        # extrapolated to the target as ~ 1/t
        own = float(np.mean(np.maximum(img2 - img * img, 0.0) / n / (ref ** 2 + 1e-2)))
        moments_est[label] = {"relmse_from_own_variance": own, "time_to_target_s": t_dev * own / args.target}
        return curve

    def plain_chunk(c, spp):
        return pi.render(scene, spp=c, first_sample=spp, accumulate=spp > 0, readback=False, graph=True).stats

    guide = G.Guide(ctx, learning_rate=1e-3, batch_size=16384, samples_per_pass=args.pool, warmup_passes=args.guide_warmup,
                    pass_paths=args.pass_paths, epochs=args.epochs)
    gstats = {}

    def guided_chunk(c, spp):
        r = pi.render_guided(scene, guide, spp=c, first_sample=spp, accumulate=spp > 0, readback=False)
        gstats.update({k: getattr(r.guide, k) for k, _ in A.bg_guide_stats._fields_})
        gstats["train_ms_total"] = gstats.get("train_ms_total", 0.0) + r.guide.train_ms
        return r.stats

    clocks = Clocks(0)
    clocks.start()
    plain_curve = progressive(plain_chunk, "plain")
    guided_curve = progressive(guided_chunk, "guided")
    clk = clocks.stop()
    pc = [(t, e) for t, e, _, _ in plain_curve]
    gc = [(t, e) for t, e, _, _ in guided_curve]
    t_plain, ext_p = _time_to(pc, args.target)
    t_guided, ext_g = _time_to(gc, args.target)
    t_eq = min(pc[-1][0], gc[-1][0])
    plain_rate = plain_curve[-1][3] * npix / plain_curve[-1][0] / 1e6
    guided_rate = guided_curve[-1][3] * npix / guided_curve[-1][0] / 1e6
    # plain samples per pixel to the target (same estimator on the CPU)
    spp_plain_target = t_plain * plain_rate * 1e6 / npix
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sdc = S.slit_room(W, H, spp=4, light_intensity=200.0) if not args.small else sd
        sdc.spp = 4
        orc, rows, nsamples, build_s = cpu_sample(sdc, args.cpu_seconds, threads)
        cv, cdt = time_cpu(orc, sdc, rows, nsamples, threads)
        cpu = {"value": spp_plain_target * npix / (cv * 1e6), "unit": "s", "cores": threads, "kind": "port",
               "msamples_per_s": cv,
               "sample": f"rows 0..{H} step {rows[2]} x {W} px x 4 spp = {nsamples} samples in {cdt:.1f} s "
                         "(oracle/, PBRT mode, bucket-fixed BVH); time = plain samples to the target / this rate"}
    wall_g = guided_curve[-1][2] * (t_guided / gc[-1][0])
    line = {
        "metric": "time-to-relMSE 1e-3 (guided)", "value": t_guided, "unit": "s", "n_gpus": 1, "steps": len(gc),
        "warmup": 0, "ms_per_step": 1e3 * gc[-1][0] / len(gc), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (network bf16)", "data": "synthetic (seeded scene generator)",
        "config": {"workload": f"slit room {W}x{H}, max depth {sd.max_depth}, {sd.ntri} triangles, {sd.nsph} "
                               f"spheres, PBRT estimator; reference {args.ref_spp} spp plain",
                   "relmse": "mean (x - ref)^2 / (ref^2 + 0.01) minus the reference's own variance term",
                   "guide": f"78 -> 4x64 -> 2 x 41 BF16 MLP (continuation and next-event heads of 8 vMF lobes), {args.pool} samples / pass of {args.pass_paths} "
                            f"paths, {args.epochs} epochs / pass, Adam lr 1e-3, batch 16384, "
                            f"{args.guide_warmup} warm-up passes"},
        "plain": {"time_to_target_s": t_plain, "extrapolated": ext_p, "msamples_per_s": plain_rate,
                  "spp_to_target": spp_plain_target, "curve": [[round(t, 4), e] for t, e in pc]},
        "guided": {"time_to_target_s": t_guided, "extrapolated": ext_g, "msamples_per_s": guided_rate,
                   "curve": [[round(t, 4), e] for t, e in gc], "stats": gstats},
        "guided_over_plain_time": t_guided / t_plain,
        "from_own_variance": dict(moments_est, guided_over_plain_time=(
            moments_est["guided"]["time_to_target_s"] / moments_est["plain"]["time_to_target_s"])),
        "equal_time": {"t_s": t_eq, "relmse_plain": _at_time(pc, t_eq) or pc[-1][1],
                       "relmse_guided": _at_time(gc, t_eq) or gc[-1][1]},
        "reference_render_s": ref_s, "reference_var_term": ref_var_term,
        "e2e": {"value": wall_g, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "note": "host wall clock of the guided calls to the target (scaled at the last checkpoint)"},
        "cpu_baseline": cpu,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    guide.close()
    scene.close()
    ctx.close()


def run_relmse(args):
    """relMSE of the stated renders against --ref-spp (default 16384) renders of the same scene and
    estimator mode: the Cornell box (256 x 256, 16 spp, depth 5) in REF_COMPAT (the reference's
    estimator over its own BVH) and PBRT mode, and the 1080p production scene (64 spp, depth 8) in
    PBRT mode.  relMSE = mean over pixels and channels of (x - ref)^2 / (ref^2 + 0.01), minus the
    reference's own expected contribution; the reference render draws disjoint sample indices."""
    from bonsai_gb300 import _abi as A
    from bonsai_gb300 import gpu as G
    from bonsai_gb300 import scenes as S
    ctx = G.Context(0)
    out = {}
    cases = [("cornell_256_16spp_ref_compat", S.cornell(256, 256, spp=16), A.BG_MODE_REF_COMPAT, A.BG_BVH_REFERENCE),
             ("cornell_256_16spp_pbrt", S.cornell(256, 256, spp=16), A.BG_MODE_PBRT, A.BG_BVH_WIDE)]
    if not args.small:
        cases.append(("production_1080p_64spp_pbrt", S.production(), A.BG_MODE_PBRT, A.BG_BVH_WIDE))
    for name, sd, mode, bvh in cases:
        W, H = sd.camera.width, sd.camera.height
        scene = G.Scene(ctx, sd, bvh)
        pi = G.PathIntegrator(sd.camera, sd.spp, sd.max_depth, sd.rr_threshold, mode=mode, seed=0)
        graph = mode == A.BG_MODE_PBRT
        t0 = time.time()
        chunk = max(1, min(args.ref_spp, (1 << 30) // (W * H)))
        for k in range(0, args.ref_spp, chunk):
            pi.render(scene, spp=min(chunk, args.ref_spp - k), first_sample=(1 << 26) + k, accumulate=k > 0,
                      readback=False, graph=graph)
        s1, s2, n = G.PathIntegrator.moments(ctx, W, H)
        nn = np.maximum(n[..., None], 1).astype(np.float64)
        ref, ref2 = s1 / nn, s2 / nn
        ref_var_term = float(np.mean(np.maximum(ref2 - ref * ref, 0.0) / nn / (ref ** 2 + 1e-2)))
        ref_s = time.time() - t0
        r = pi.render(scene, graph=graph)
        s1, s2, n = G.PathIntegrator.moments(ctx, W, H)
        img = s1 / np.maximum(n[..., None], 1)
        out[name] = {"relmse": _relmse(img, ref, ref_var_term), "relmse_uncorrected": _relmse(img, ref, 0.0),
                     "reference_var_term": ref_var_term, "spp": sd.spp, "reference_spp": args.ref_spp,
                     "size": [W, H], "reference_render_s": ref_s, "error_word": int(r.stats.error_word)}
        print(name, json.dumps(out[name]), flush=True)
        scene.close()
    print(json.dumps({"metric": "relMSE vs a high-spp render", "unit": "relMSE", "results": out,
                      "relmse": "mean (x - ref)^2 / (ref^2 + 0.01) minus the reference's own variance term"}),
          flush=True)
    ctx.close()


def _random_guide_data(n: int, seed: int):
    """Seeded synthetic training samples / queries with the value ranges the renderer produces."""
    rng = np.random.default_rng(seed)

    def unit(k):
        v = rng.normal(size=(k, 3))
        return v / np.linalg.norm(v, axis=1, keepdims=True)
    s = np.zeros((n, 16), np.float32)
    s[:, 0:3] = rng.random((n, 3))
    s[:, 3:6] = unit(n)
    s[:, 6:9] = unit(n)
    s[:, 9:12] = unit(n)
    s[:, 12] = rng.exponential(0.3, n)
    s[:, 13] = rng.lognormal(0.0, 1.0, n)
    s[:, 14] = np.where(rng.random(n) < 0.9, 0.0, rng.lognormal(0.0, 1.0, n))
    return s


def run_guided_pass(args):
    """Cost of one pass of the guiding workload's slit room (1280x720, 4 spp, depth 10): plain
    (per-launch, no graph, as the guided passes launch), guided with the network frozen, and guided
    with recording and training, after the network has trained for 24 passes.  Three repetitions;
    with --profile the last one runs inside a profiler window (cuProfilerStart / cuProfilerStop) for
    `ncu --profile-from-start off`."""
    import ctypes
    from bonsai_gb300 import _abi as A
    from bonsai_gb300 import gpu as G
    from bonsai_gb300 import scenes as S
    sd = S.slit_room(light_intensity=200.0)
    ctx = G.Context(0)
    scene = G.Scene(ctx, sd, A.BG_BVH_WIDE)
    pi = G.PathIntegrator(sd.camera, 1, sd.max_depth, sd.rr_threshold, mode=A.BG_MODE_PBRT, seed=11)
    g = G.Guide(ctx, learning_rate=1e-3, batch_size=16384, samples_per_pass=1 << 18, warmup_passes=8,
                pass_paths=1 << 22, epochs=args.epochs, no_fallback=True)
    pi.render_guided(scene, g, spp=4 * 24, first_sample=1 << 20, readback=False)
    fz = G.Guide(ctx, batch_size=16384, samples_per_pass=1 << 18, warmup_passes=0, pass_paths=1 << 22,
                 no_fallback=True, no_train=True)
    fz.params = g.params
    cu = ctypes.CDLL("libcuda.so.1") if args.profile else None
    ms = {"plain": [], "frozen": [], "training": [], "training_train": []}
    for rep in range(3):
        if cu is not None and rep == 2:
            cu.cuProfilerStart()
        ms["plain"].append(pi.render(scene, spp=4, first_sample=rep * 4, readback=False, graph=False).stats.device_ms)
        ms["frozen"].append(pi.render_guided(scene, fz, spp=4, first_sample=rep * 4, readback=False).stats.device_ms)
        r = pi.render_guided(scene, g, spp=4, first_sample=(1 << 22) + rep * 4, readback=False)
        ms["training"].append(r.stats.device_ms)
        ms["training_train"].append(r.guide.train_ms)
        if cu is not None and rep == 2:
            cu.cuProfilerStop()
    med = {k: float(np.median(v)) for k, v in ms.items()}
    print(json.dumps({"metric": "guided pass device time", "unit": "ms", "plain_ms": med["plain"],
                      "frozen_ms": med["frozen"], "training_ms": med["training"],
                      "training_train_ms": med["training_train"],
                      "frozen_over_plain": med["frozen"] / med["plain"],
                      "training_over_plain": med["training"] / med["plain"], "profiled": bool(args.profile),
                      "config": {"workload": f"slit room {sd.camera.width}x{sd.camera.height}, 4 spp per pass, max "
                                             f"depth {sd.max_depth}; guide trained 24 passes, {args.epochs} epochs "
                                             "of a 2^18-sample pool per training pass"}}))
    fz.close()
    g.close()
    scene.close()
    ctx.close()


def run_guide_mlp(args):
    """The guiding network alone: device time of a training step (forward + backward + Adam on one
    16384-sample batch) and of inference over 2^20 queries.  FLOPs are the network's algorithmic
    count: 22,528 multiply-adds per inference (78 -> 4 x 64 -> 2 x 41) = 45,056 FLOP, 3x that per
    training sample; the denominator is the measured cuBLAS BF16 peak."""
    from bonsai_gb300 import gpu as G
    ctx = G.Context(0)
    g = G.Guide(ctx, batch_size=16384, samples_per_pass=1 << 18)
    data = _random_guide_data(1 << 20, 5)
    clocks = Clocks(0)
    clocks.start()
    step_ms, infer_ms = g.time(data[:16384], data[:, :9], reps=max(args.steps, 3))
    clk = clocks.stop()
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("bf16_tflops", 1900.0))
    fl_inf = 2 * (78 * 64 + 3 * 64 * 64 + 64 * 82)
    train_tf = 3 * fl_inf * 16384 / (step_ms / 1e3) / 1e12
    infer_tf = fl_inf * len(data) / (infer_ms / 1e3) / 1e12
    print(json.dumps({
        "metric": "guiding network throughput", "value": len(data) / (infer_ms / 1e3) / 1e6, "unit": "Mqueries/s",
        "n_gpus": 1, "steps": max(args.steps, 3), "higher_is_better": True, "dtype": "bf16 (fp32 accumulate)",
        "train_step_ms": step_ms, "train_samples_per_s": 16384 / (step_ms / 1e3), "infer_ms_2^20": infer_ms,
        "roofline": {"bound": "tensor", "unit": "TFLOP/s", "peak": peak,
                     "peak_source": "measured" if peaks else "fallback",
                     "train": {"achieved": train_tf, "frac": train_tf / peak},
                     "infer": {"achieved": infer_tf, "frac": infer_tf / peak}},
        "clocks": clk}), flush=True)
    g.close()
    ctx.close()


def run_batch(args):
    """Uneven multi-scene batch: 256 seeded scenes (1k..500k triangles, 128^2..512^2 / 640x360,
    4..64 spp, depth 4..10) rendered by bg_render_batch, whose paths of all scenes share one
    wavefront; value = aggregate Msamples/s of the batch (device time, L2 flushed before every step).
    Compared with rendering the same scenes one after another through bg_render (graph-captured),
    for all scenes and for the small ones (<= 256^2 pixels, <= 16 spp).  Time to relMSE 1e-3 per
    scene from each scene's relative variance per sample (batch film moments) and its measured
    one-at-a-time rate, and for the whole batch at its aggregate rate.  Guided arm: --guided-scenes
    scenes spread over the batch's sizes, each with its own network trained online
    (--guided-train-passes passes), then time to target = relvar x ms per spp of the frozen network
    against the plain render of the same scene."""
    from bonsai_gb300 import _abi as A
    from bonsai_gb300 import gpu as G
    from bonsai_gb300 import scenes as S
    nsc = 32 if args.small else 256
    t0 = time.time()
    sds = S.uneven_batch(nsc)
    gen_s = time.time() - t0
    ctx = G.Context(0)
    t0 = time.time()
    scenes = [G.Scene(ctx, sd, A.BG_BVH_WIDE) for sd in sds]
    build_s = time.time() - t0
    jobs = [G.BatchJob(sc, sd.camera, sd.spp, sd.max_depth, seed=k) for k, (sc, sd) in enumerate(zip(scenes, sds))]
    samples = sum(sd.camera.width * sd.camera.height * sd.spp for sd in sds)
    for _ in range(args.warmup):
        G.render_batch(ctx, jobs, readback=False)
    clocks = Clocks(0)
    clocks.start()
    dev_ms, launches = 0.0, 0
    for _ in range(args.steps):
        ctx.flush_l2()
        _, st = G.render_batch(ctx, jobs, readback=False)
        dev_ms += st.device_ms
        launches += st.launches
    clk = clocks.stop()
    value = args.steps * samples / (dev_ms / 1e3) / 1e6
    t0 = time.time()
    for _ in range(args.steps):
        imgs, _ = G.render_batch(ctx, jobs, readback=True)
    e2e = args.steps * samples / (time.time() - t0) / 1e6
    d2h = sum(im.nbytes for im in imgs)
    # per-scene relative variance per sample (relMSE denominator as in the guiding workload) from the
    # batch film's moments: relMSE after n samples per pixel = relvar / n
    G.render_batch(ctx, jobs, readback=False)
    npix = [sd.camera.width * sd.camera.height for sd in sds]
    s1, s2, cnt = G.PathIntegrator.moments(ctx, sum(npix), 1)
    s1, s2, cnt = s1.reshape(-1, 3), s2.reshape(-1, 3), cnt.reshape(-1, 1).astype(np.float64)
    m = s1 / cnt
    var = np.maximum(s2 / cnt - m * m, 0.0)
    relvar, p0 = [], 0
    for n in npix:
        relvar.append(float(np.mean(var[p0:p0 + n] / (m[p0:p0 + n] ** 2 + 1e-2))))
        p0 += n
    spp_target = [rv / args.target for rv in relvar]
    # the same scenes one render at a time (graph-captured wavefront per scene)
    seq_ms = 0.0
    seq_each = []
    ctx.flush_l2()
    for j in jobs:
        pi = G.PathIntegrator(j.camera, j.spp, j.max_depth, mode=A.BG_MODE_PBRT, seed=j.seed)
        pi.render(j.scene, readback=False, graph=True)  # capture
        ms = pi.render(j.scene, readback=False, graph=True).stats.device_ms
        seq_ms += ms
        seq_each.append(ms)
    batch_rate = samples / (dev_ms / args.steps / 1e3)
    # time to relMSE 1e-3 in every scene: one batch delivering every scene's samples to the target
    # at the batch's aggregate rate, against one-at-a-time renders at each scene's measured rate
    tt_batch = sum(st * n for st, n in zip(spp_target, npix)) / batch_rate
    tt_seq_each = [st * ms / 1e3 / j.spp for st, ms, j in zip(spp_target, seq_each, jobs)]
    # the small scenes (<= 256 x 256 pixels and <= 16 spp), where a one-scene render cannot fill the GPU
    small = [k for k, sd in enumerate(sds) if npix[k] <= 256 * 256 and sd.spp <= 16]
    small_res = None
    if small:
        sjobs = [jobs[k] for k in small]
        ssamples = sum(npix[k] * sds[k].spp for k in small)
        G.render_batch(ctx, sjobs, readback=False)
        sms = 0.0
        for _ in range(args.steps):
            ctx.flush_l2()
            sms += G.render_batch(ctx, sjobs, readback=False)[1].device_ms
        sms /= args.steps
        sseq = sum(seq_each[k] for k in small)
        small_res = {"scenes": len(small), "samples": ssamples, "batch_ms": sms, "sequential_ms": sseq,
                     "batch_msamples_per_s": ssamples / (sms / 1e3) / 1e6,
                     "sequential_msamples_per_s": ssamples / (sseq / 1e3) / 1e6,
                     "batch_over_sequential": sseq / sms}
    # guided arm on a spread of scenes: each scene's guide trains online, then its frozen network
    # renders the scene's spp; time to target = relvar / target x ms per spp, against plain
    guided = []
    if args.guided_scenes > 0:
        order = sorted(range(nsc), key=lambda k: npix[k] * sds[k].spp)
        picks = [order[int(i * (nsc - 1) / max(args.guided_scenes - 1, 1))] for i in range(args.guided_scenes)]
        for k in picks:
            j, sd = jobs[k], sds[k]
            pi = G.PathIntegrator(j.camera, j.spp, j.max_depth, mode=A.BG_MODE_PBRT, seed=j.seed)
            g = G.Guide(ctx, learning_rate=1e-3, batch_size=16384, samples_per_pass=1 << 18, warmup_passes=4,
                        pass_paths=1 << 22, epochs=2, no_fallback=True)
            pass_spp = max(1, (1 << 22) // npix[k])
            r = pi.render_guided(j.scene, g, spp=pass_spp * args.guided_train_passes, first_sample=1 << 22,
                                 readback=False)
            fz = G.Guide(ctx, batch_size=16384, samples_per_pass=1 << 18, warmup_passes=0, pass_paths=1 << 22,
                         no_fallback=True, no_train=True)
            fz.params = g.params
            rg = pi.render_guided(j.scene, fz, spp=j.spp, first_sample=0, readback=False)
            g1, g2, gn = G.PathIntegrator.moments(ctx, sd.camera.width, sd.camera.height)
            gn = gn[..., None].astype(np.float64)
            gm = g1 / gn
            rv_g = float(np.mean(np.maximum(g2 / gn - gm * gm, 0.0) / (gm ** 2 + 1e-2)))
            ms_g = rg.stats.device_ms / j.spp
            ms_p = seq_each[k] / j.spp
            guided.append({"scene": k, "pixels": npix[k], "spp": j.spp, "triangles": sd.ntri,
                           "relvar_plain": relvar[k], "relvar_guided": rv_g,
                           "ms_per_spp_plain": ms_p, "ms_per_spp_guided": ms_g,
                           "time_to_target_plain_s": relvar[k] / args.target * ms_p / 1e3,
                           "time_to_target_guided_s": rv_g / args.target * ms_g / 1e3,
                           "guided_over_plain_time": (rv_g * ms_g) / (relvar[k] * ms_p) if relvar[k] > 0 else None,
                           "training_s": (r.guide.render_ms + r.guide.train_ms) / 1e3})
            fz.close()
            g.close()
    print(json.dumps({
        "metric": "Msamples/s (uneven batch)", "value": value, "unit": "Msamples/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
        "config": {"workload": f"uneven batch of {nsc} scenes (scenes.uneven_batch(seed 5)): "
                               f"{sum(sd.ntri for sd in sds)} triangles, {samples} samples per step",
                   "l2": "flushed before every step"},
        "e2e": {"value": e2e, "unit": "Msamples/s", "h2d_bytes_per_step": nsc * 368, "d2h_bytes_per_step": d2h,
                "note": "h2d = the 368-byte scene table entry per scene uploaded by every call"},
        "gpu_launches": launches,
        "sequential_msamples_per_s": samples / (seq_ms / 1e3) / 1e6,
        "batch_over_sequential": (samples / (dev_ms / args.steps / 1e3)) / (samples / (seq_ms / 1e3)),
        "small_scenes": small_res,
        "time_to_relmse": {"target": args.target,
                           "definition": "relMSE after n spp = relvar / n, relvar = mean over pixels and channels of "
                                         "var / (mean^2 + 0.01) from the batch film's moments",
                           "all_scenes_batch_s": tt_batch, "all_scenes_sequential_s": sum(tt_seq_each),
                           "per_scene": [{"scene": k, "pixels": npix[k], "spp": sds[k].spp, "triangles": sds[k].ntri,
                                          "relvar": round(relvar[k], 4), "spp_to_target": round(spp_target[k], 1),
                                          "sequential_s": round(tt_seq_each[k], 4)} for k in range(nsc)]},
        "guided_scenes": guided,
        "scene_generation_s": gen_s, "upload_and_bvh_build_s": build_s, "clocks": clk}), flush=True)
    for sc in scenes:
        sc.close()
    ctx.close()


def main():
    args = parse()
    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload == "guide-mlp":
        run_guide_mlp(args)
        return
    if args.workload == "raysoup":
        run_raysoup(args)
        return
    if args.workload == "guiding":
        run_guiding(args)
        return
    if args.workload == "relmse":
        run_relmse(args)
        return
    if args.workload == "guided-pass":
        run_guided_pass(args)
        return
    if args.workload in ("whitted", "direct", "example"):
        run_integrators(args)
        return
    if args.profile:
        run_profile(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

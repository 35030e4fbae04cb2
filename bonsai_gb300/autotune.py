"""Autotuner for the wavefront launch parameters (bg_tuning).

Tunes, by coordinate descent on short renders of the actual scene (device-timed with the
library's CUDA events, L2 flushed before each trial):
  refill        - traversal: lanes a warp lets go idle before it fetches new rays (32 = whole warp)
  blocks_per_sm - persistent grid of the wavefront stages
  wave_paths    - paths per wave (queue capacity)
  sort_rays     - bin each bounce's extension rays by direction octant and origin cell
  concurrent_shade - run a bounce's material-class shade kernels side by side
and, by tune_layout, the traversal node width: the scene's BVH built 8-wide (BG_BVH_WIDE) and
2-wide (BG_BVH_WIDE2), each timed on the same trial render.
The result is cached as JSON keyed by GPU name, scene signature and render settings
(default ~/.cache/bonsai_gb300/tuning.json, or $BONSAI_TUNING_CACHE).
"""
from __future__ import annotations

import ctypes as C
import json
import os
from pathlib import Path

from . import _abi as A

REFILL = [32, 16, 8, 4]
BLOCKS = [4, 8, 16]
WAVES = [1 << 20, 1 << 21, 1 << 22, 1 << 23, 1 << 24, 1 << 25]
SORT = [0, 1]
CONCURRENT = [1, 0]


def cache_path() -> Path:
    p = os.environ.get("BONSAI_TUNING_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "bonsai_gb300" / "tuning.json"


def _gpu_name() -> str:
    try:
        import subprocess
        return subprocess.run(["nvidia-smi", "--query-gpu=name", "--format=csv,noheader", "-i", "0"],
                              capture_output=True, text=True, timeout=10).stdout.strip() or "unknown"
    except Exception:
        return "unknown"


def key_of(sd, spp: int) -> str:
    c = sd.camera
    return f"{_gpu_name()}|tri{sd.ntri}|sph{sd.nsph}|{c.width}x{c.height}|depth{sd.max_depth}|spp{spp}|v4"


def get(ctx) -> A.bg_tuning:
    t = A.bg_tuning()
    ctx.check(ctx.lib.bg_get_tuning(ctx.h, C.byref(t)))
    return t


def set_(ctx, refill: int, blocks: int, wave: int, sort_rays: int = 0, concurrent_shade: int = 1):
    t = A.bg_tuning()
    t.refill, t.blocks_per_sm, t.wave_paths = refill, blocks, wave
    t.flags = ((A.BG_TUNE_SORT_RAYS if sort_rays else 0) | A.BG_TUNE_TILE_PIXELS |
               (A.BG_TUNE_CONCURRENT_SHADE if concurrent_shade else 0))
    ctx.check(ctx.lib.bg_set_tuning(ctx.h, C.byref(t)))


def _trial(ctx, scene, integrator, spp: int, reps: int = 3) -> float:
    best = float("inf")
    for _ in range(reps):
        ctx.flush_l2()
        r = integrator.render(scene, readback=False, spp=spp)
        best = min(best, r.stats.device_ms)
    return best


def tune(ctx, scene, integrator, spp: int = 4, use_cache: bool = True, verbose: bool = False) -> dict:
    """Returns {"refill", "blocks_per_sm", "wave_paths", "ms", "trials"} and applies it to ctx."""
    sd = scene.sd
    key = key_of(sd, spp)
    path = cache_path()
    cache = {}
    if use_cache and path.exists():
        try:
            cache = json.loads(path.read_text())
        except ValueError:
            cache = {}
    if use_cache and key in cache:
        c = cache[key]
        set_(ctx, c["refill"], c["blocks_per_sm"], c["wave_paths"], c.get("sort_rays", 0), c.get("concurrent_shade", 1))
        return dict(c, cached=True)
    cur = {"refill": 32, "blocks_per_sm": 8, "wave_paths": 1 << 22, "sort_rays": 0, "concurrent_shade": 1}
    trials = []

    def run(cfg, tspp):
        set_(ctx, cfg["refill"], cfg["blocks_per_sm"], cfg["wave_paths"], cfg["sort_rays"], cfg["concurrent_shade"])
        integrator.render(scene, readback=False, spp=1)  # allocate / warm
        ms = _trial(ctx, scene, integrator, tspp)
        trials.append(dict(cfg, ms=ms, spp=tspp))
        if verbose:
            print("autotune", cfg, f"{ms:.2f} ms")
        return ms

    # a wave larger than a trial's paths changes nothing, so wave sizes are compared on trials of at
    # least two of the largest waves (otherwise the choice among them is noise)
    npix = sd.camera.width * sd.camera.height
    wave_spp = max(spp, -(-2 * max(WAVES) // npix))
    best_ms = float("inf")
    for name, values in (("refill", REFILL), ("blocks_per_sm", BLOCKS), ("wave_paths", WAVES), ("sort_rays", SORT),
                         ("concurrent_shade", CONCURRENT)):
        tspp = wave_spp if name == "wave_paths" else spp
        best_ms = run(cur, tspp)
        for v in values:
            if v == cur[name]:
                continue
            cfg = dict(cur, **{name: v})
            ms = run(cfg, tspp)
            # a larger wave wins ties within 0.5% (fewer wave tails at the render's full spp)
            if ms < best_ms * (0.995 if name != "wave_paths" or v < cur[name] else 1.005):
                best_ms, cur = ms, cfg
    set_(ctx, cur["refill"], cur["blocks_per_sm"], cur["wave_paths"], cur["sort_rays"], cur["concurrent_shade"])
    result = dict(cur, ms=best_ms, trials=trials)
    if use_cache:
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            cache[key] = {k: result[k] for k in ("refill", "blocks_per_sm", "wave_paths", "sort_rays", "concurrent_shade",
                                                 "ms")}
            path.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    return result


LAYOUTS = [A.BG_BVH_WIDE, A.BG_BVH_WIDE2]  # 8-wide compressed, 2-wide


def tune_layout(ctx, sd, integrator, spp: int = 4, use_cache: bool = True, verbose: bool = False):
    """Traversal node width for scene data `sd`: builds the BVH in each wide layout, times a trial
    render of each at the context's current launch shape, keeps the faster.  Returns (scene, info)
    with the kept scene built (the other one is closed); info = {"layout", "ms", "trials", "cached"}.
    The choice is cached like the launch parameters."""
    from . import gpu as G
    key = "layout|" + key_of(sd, spp)
    path = cache_path()
    cache = {}
    if use_cache and path.exists():
        try:
            cache = json.loads(path.read_text())
        except ValueError:
            cache = {}
    if use_cache and key in cache:
        c = cache[key]
        return G.Scene(ctx, sd, int(c["layout"])), dict(c, cached=True)
    best, best_ms, trials = None, float("inf"), []
    for layout in LAYOUTS:
        sc = G.Scene(ctx, sd, layout)
        integrator.render(sc, readback=False, spp=1)  # warm
        ms = _trial(ctx, sc, integrator, spp)
        trials.append({"layout": int(layout), "ms": ms})
        if verbose:
            print("autotune layout", layout, f"{ms:.2f} ms")
        if ms < best_ms:
            if best is not None:
                best.close()
            best, best_ms = sc, ms
        else:
            sc.close()
    info = {"layout": int(best.layout), "ms": best_ms, "trials": trials}
    if use_cache:
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            cache[key] = {"layout": info["layout"], "ms": best_ms}
            path.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    return best, dict(info, cached=False)

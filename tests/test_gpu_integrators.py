"""The Whitted and direct-lighting integrators (src/integrators/{whitted,direct}.rs): device renders
against the CPU oracle's recursive restatement (same random numbers per ray-tree node), in both
estimator modes, over the three BVH layouts, on a room with a glass sphere (the specular
recursion) and textured walls (ray differentials carried through specular bounces)."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from bonsai_gb300 import _abi as A
from bonsai_gb300 import gpu as G
from bonsai_gb300 import scenes as S

from .parity import compare_renders

pytestmark = pytest.mark.gpu

Z3_FRAC = 0.01
KINDS = [("whitted", A.BG_INTEGRATOR_WHITTED, 0), ("direct_all", A.BG_INTEGRATOR_DIRECT, A.BG_LIGHT_UNIFORM_ALL),
         ("direct_one", A.BG_INTEGRATOR_DIRECT, A.BG_LIGHT_UNIFORM_ONE)]


def glass_room(w=40, h=40, spp=16, max_depth=5, textured=True):
    """The textured room (or the plain Cornell box) with its conductor sphere turned to glass."""
    sd = S.textured_room(w, h, spp=spp, max_depth=max_depth) if textured else S.cornell(w, h, spp, max_depth)
    mats = list(sd.materials) + [S.material(S.DIELECTRIC, ior=1.5)]
    sd.materials = np.stack(mats)
    sd.spheres = sd.spheres.copy()
    sd.spheres[1]["material_id"] = len(mats) - 1
    return sd


def _integrator(cls_kind, strategy, cam, spp, depth, mode):
    if cls_kind == A.BG_INTEGRATOR_WHITTED:
        return G.WhittedIntegrator(cam, spp, depth, mode=mode)
    return G.DirectLightingIntegrator(cam, spp, depth, strategy, mode=mode)


def _pair(ctx, sd, kind, strategy, mode, bvh, spp):
    o = O.OracleScene(sd, fixed_bvh=True).render(mode, spp=spp, integrator=kind, light_strategy=strategy)
    sc = G.Scene(ctx, sd, bvh)
    try:
        r = _integrator(kind, strategy, sd.camera, spp, sd.max_depth, mode).render(sc)
    finally:
        sc.close()
    s1, s2, n = G.PathIntegrator.moments(ctx, sd.camera.width, sd.camera.height)
    assert (n == spp).all()
    return r, o, compare_renders(s1, s2, n, o["sum"], o["sumsq"], np.full(n.shape, spp))


@pytest.mark.parametrize("name,kind,strategy", KINDS)
@pytest.mark.parametrize("bvh", [A.BG_BVH_WIDE, A.BG_BVH_WIDE2, A.BG_BVH_REFERENCE_FIXED])
def test_pbrt_matches_oracle(gpu_ctx, name, kind, strategy, bvh):
    sd = glass_room()
    r, o, cmp = _pair(gpu_ctx, sd, kind, strategy, A.BG_MODE_PBRT, bvh, 16)
    print(name, cmp)
    assert r.stats.error_word == 0
    assert cmp["frac_z3"] <= Z3_FRAC
    assert cmp["frac_close"] >= 0.9
    np.testing.assert_allclose(r.rgb.mean(), o["rgb"].mean(), rtol=2e-3)


@pytest.mark.parametrize("name,kind,strategy", KINDS)
def test_ref_compat_matches_oracle(gpu_ctx, name, kind, strategy):
    sd = glass_room(textured=False)
    r, o, cmp = _pair(gpu_ctx, sd, kind, strategy, A.BG_MODE_REF_COMPAT, A.BG_BVH_REFERENCE_FIXED, 16)
    print(name, cmp)
    assert cmp["frac_z3"] <= Z3_FRAC
    assert cmp["frac_close"] >= 0.9


def _sphere_pixels(sd):
    """Pixels whose camera ray hits the glass sphere (sphere 1), from the oracle's ray queries."""
    cam = sd.camera
    ys, xs = np.mgrid[0:cam.height, 0:cam.width]
    rays = np.zeros(cam.width * cam.height, S.RAY_DT)
    for i, (x, y) in enumerate(zip(xs.ravel(), ys.ravel())):
        r = O.camera_ray(cam, x + 0.5, y + 0.5)
        rays[i]["org"], rays[i]["dir"], rays[i]["tmax"] = r[:3], r[3:], np.inf
    hits = O.OracleScene(sd).trace(rays)
    m = (hits["prim"] == sd.ntri + 1).reshape(cam.height, cam.width)
    # interior pixels only: the samples of an edge pixel also see what lies around the sphere
    inner = m.copy()
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            inner &= np.roll(np.roll(m, dy, 0), dx, 1)
    return inner


def test_specular_recursion_runs_in_pbrt_mode_only(gpu_ctx):
    """The glass splits into SpecularReflection + SpecularTransmission in PBRT mode, so Whitted sees
    the room through it; the reference's own FresnelSpecular lobe matches neither specular query
    (bsdf.rs matches_flags), so in REF_COMPAT mode the glass stays black."""
    sd = glass_room(textured=False)
    mask = _sphere_pixels(sd)
    assert mask.sum() > 10
    out = {}
    for mode, bvh in ((A.BG_MODE_PBRT, A.BG_BVH_WIDE), (A.BG_MODE_REF_COMPAT, A.BG_BVH_REFERENCE_FIXED)):
        sc = G.Scene(gpu_ctx, sd, bvh)
        try:
            out[mode] = G.WhittedIntegrator(sd.camera, 16, 5, mode=mode).render(sc).rgb
        finally:
            sc.close()
    assert out[A.BG_MODE_PBRT][mask].mean() > 0.05
    assert out[A.BG_MODE_REF_COMPAT][mask].max() == 0.0


def test_depth_limits(gpu_ctx):
    sd = glass_room(8, 8, textured=False)
    sc = G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)
    try:
        with pytest.raises(RuntimeError, match="max_depth"):
            G.WhittedIntegrator(sd.camera, 1, 31).render(sc)
        r = G.WhittedIntegrator(sd.camera, 1, 30).render(sc)  # deepest allowed tree
        assert r.stats.error_word == 0
        o = A.bg_render_opts()
        assert r.stats.samples == 64 and o.integrator == 0
    finally:
        sc.close()


def test_small_tree_waves_match_large_ones(gpu_ctx):
    """The tree wavefront renders in waves of at most bg_tuning.wave_paths samples; a wave whose
    ray trees outgrow a level queue is discarded and rendered again in halves.  Tiny waves over
    deep glass trees (reached only through the halving when a wave overflows) give the film of one
    large wave up to float summation order."""
    sd = glass_room(48, 48, spp=8, max_depth=12, textured=False)
    sd.spheres = sd.spheres.copy()
    sd.spheres[0]["material_id"] = sd.spheres[1]["material_id"]  # both spheres glass
    out = []
    saved = A.bg_tuning()
    gpu_ctx.check(gpu_ctx.lib.bg_get_tuning(gpu_ctx.h, C.byref(saved)))
    sc = G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)
    try:
        for wave in (1 << 20, 1024):
            t = A.bg_tuning.from_buffer_copy(bytes(saved))
            t.wave_paths = wave
            gpu_ctx.check(gpu_ctx.lib.bg_set_tuning(gpu_ctx.h, C.byref(t)))
            r = G.WhittedIntegrator(sd.camera, 8, 12).render(sc)
            assert r.stats.error_word == 0
            out.append((r.rgb, r.stats.launches))
    finally:
        gpu_ctx.check(gpu_ctx.lib.bg_set_tuning(gpu_ctx.h, C.byref(saved)))
        sc.close()
    (a, la), (b, lb) = out
    assert lb > la  # many more waves
    np.testing.assert_allclose(a, b, rtol=1e-4, atol=1e-5)

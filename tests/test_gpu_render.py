"""Oracle (b): per-pixel render parity of the device path tracer against the CPU oracle.

Both sides draw the same counter-based random numbers (Philox4x32-10 keyed by pixel, sample and
dimension), so most paths are identical; transcendental-function ulps, fma-based error-free
products (the reference's f64 spots) and the wide BVH's tie order separate a few.  Bar: fraction
of pixel channels more than 3 combined standard errors apart <= 1% (a Gaussian gives 0.27%).
"""
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


def _render_pair(ctx, sd, mode, bvh, spp, seed=0):
    orc = O.OracleScene(sd, fixed_bvh=(bvh != A.BG_BVH_REFERENCE))
    o = orc.render(mode, spp=spp, seed=seed)
    sc = G.Scene(ctx, sd, bvh)
    pi = G.PathIntegrator(sd.camera, spp, sd.max_depth, sd.rr_threshold, mode=mode, seed=seed)
    r = pi.render(sc)
    s1, s2, n = G.PathIntegrator.moments(ctx, sd.camera.width, sd.camera.height)
    assert (n == spp).all()
    cmp = compare_renders(s1, s2, n, o["sum"], o["sumsq"], np.full(n.shape, spp))
    return r, o, cmp


def test_cornell_ref_compat(gpu_ctx):
    sd = S.cornell(64, 64)
    r, o, cmp = _render_pair(gpu_ctx, sd, A.BG_MODE_REF_COMPAT, A.BG_BVH_REFERENCE, 16)
    print(cmp)
    assert cmp["frac_z3"] <= Z3_FRAC
    assert cmp["frac_close"] >= 0.9
    assert r.stats.error_word == 0


@pytest.mark.parametrize("bvh", [A.BG_BVH_WIDE, A.BG_BVH_WIDE2, A.BG_BVH_REFERENCE_FIXED])
def test_cornell_pbrt(gpu_ctx, bvh):
    sd = S.cornell(64, 64)
    r, o, cmp = _render_pair(gpu_ctx, sd, A.BG_MODE_PBRT, bvh, 16)
    print(cmp)
    assert cmp["frac_z3"] <= Z3_FRAC
    assert cmp["frac_close"] >= 0.9
    np.testing.assert_allclose(r.rgb.mean(), o["rgb"].mean(), rtol=1e-3)


@pytest.mark.parametrize("bvh", [A.BG_BVH_WIDE, A.BG_BVH_WIDE2])
def test_production_small_pbrt(gpu_ctx, bvh):
    sd = S.production(96, 54, spp=4, n_ico=6, ico_level=3, n_spheres=300)
    r, o, cmp = _render_pair(gpu_ctx, sd, A.BG_MODE_PBRT, bvh, 4)
    print(cmp)
    assert cmp["frac_z3"] <= Z3_FRAC
    assert cmp["frac_close"] >= 0.8


@pytest.mark.parametrize("mode,bvh", [(A.BG_MODE_PBRT, A.BG_BVH_WIDE), (A.BG_MODE_REF_COMPAT, A.BG_BVH_REFERENCE)])
def test_quadric_box(gpu_ctx, mode, bvh):
    sd = S.quadric_box(48, 48, spp=8)
    r, o, cmp = _render_pair(gpu_ctx, sd, mode, bvh, 8)
    print(cmp)
    assert cmp["frac_z3"] <= Z3_FRAC
    assert cmp["frac_close"] >= 0.9


def test_graph_replay_matches_launches(gpu_ctx):
    sd = S.production(96, 54, spp=4, n_ico=6, ico_level=3, n_spheres=300)
    sc = G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)
    pi = G.PathIntegrator(sd.camera, 4, sd.max_depth, sd.rr_threshold, mode=A.BG_MODE_PBRT, seed=3)
    from bonsai_gb300 import autotune
    autotune.set_(gpu_ctx, 32, 8, 8192)  # several waves per render
    try:
        plain = pi.render(sc)
        for first in (0, 4):  # the captured graph is reused; first_sample travels on the device
            g = pi.render(sc, graph=True, first_sample=first)
            ref = plain if first == 0 else pi.render(sc, first_sample=first)
            np.testing.assert_allclose(g.rgb, ref.rgb, rtol=1e-6, atol=1e-7)
            assert g.stats.launches > 4 * (sd.max_depth + 1)
    finally:
        autotune.set_(gpu_ctx, 32, 8, 1 << 22)


def test_ray_binning_keeps_every_path(gpu_ctx):
    """BG_TUNE_SORT_RAYS only reorders the extension queue: every path, and so the film, is the same."""
    from bonsai_gb300 import autotune
    sd = S.production(160, 90, spp=4, max_depth=6, n_ico=4, ico_level=3, n_spheres=100)
    sc = G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)
    old = autotune.get(gpu_ctx)
    try:
        pi = G.PathIntegrator(sd.camera, sd.spp, sd.max_depth, mode=A.BG_MODE_PBRT, seed=4)
        films = []
        for flags in (0, A.BG_TUNE_SORT_RAYS):
            t = A.bg_tuning()
            t.wave_paths, t.blocks_per_sm, t.refill, t.flags = 1 << 14, old.blocks_per_sm, old.refill, flags
            gpu_ctx.check(gpu_ctx.lib.bg_set_tuning(gpu_ctx.h, C.byref(t)))
            r = pi.render(sc)
            assert r.stats.error_word == 0
            films.append((r.rgb, G.PathIntegrator.moments(gpu_ctx, sd.camera.width, sd.camera.height)))
        (rgb0, (a1, a2, an)), (rgb1, (b1, b2, bn)) = films
        np.testing.assert_array_equal(an, bn)
        np.testing.assert_allclose(a1, b1, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(a2, b2, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(rgb0, rgb1, rtol=1e-6, atol=1e-6)
    finally:
        gpu_ctx.check(gpu_ctx.lib.bg_set_tuning(gpu_ctx.h, C.byref(old)))
        sc.close()


def test_concurrent_shading_keeps_every_path(gpu_ctx):
    """BG_TUNE_CONCURRENT_SHADE runs a bounce's material-class shade kernels side by side: only the
    order of queue appends and film sums changes, so the films agree to rounding of the sums."""
    sd = S.production(160, 90, spp=4, max_depth=6, n_ico=4, ico_level=3, n_spheres=100)
    sc = G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)
    saved = A.bg_tuning()
    gpu_ctx.check(gpu_ctx.lib.bg_get_tuning(gpu_ctx.h, C.byref(saved)))
    try:
        pi = G.PathIntegrator(sd.camera, sd.spp, sd.max_depth, mode=A.BG_MODE_PBRT, seed=6)
        films = []
        for flags in (A.BG_TUNE_TILE_PIXELS, A.BG_TUNE_TILE_PIXELS | A.BG_TUNE_CONCURRENT_SHADE):
            t = A.bg_tuning.from_buffer_copy(bytes(saved))
            t.wave_paths, t.flags = 1 << 14, flags  # several waves per render
            gpu_ctx.check(gpu_ctx.lib.bg_set_tuning(gpu_ctx.h, C.byref(t)))
            for graph in (False, True):
                r = pi.render(sc, graph=graph)
                assert r.stats.error_word == 0
                films.append(G.PathIntegrator.moments(gpu_ctx, sd.camera.width, sd.camera.height))
        a1, a2, an = films[0]
        for b1, b2, bn in films[1:]:
            np.testing.assert_array_equal(an, bn)
            np.testing.assert_allclose(a1, b1, rtol=1e-12, atol=1e-12)
            np.testing.assert_allclose(a2, b2, rtol=1e-12, atol=1e-12)
    finally:
        gpu_ctx.check(gpu_ctx.lib.bg_set_tuning(gpu_ctx.h, C.byref(saved)))
        sc.close()


def _with_flags(ctx, flags, fn):
    saved = A.bg_tuning()
    ctx.check(ctx.lib.bg_get_tuning(ctx.h, C.byref(saved)))
    t = A.bg_tuning.from_buffer_copy(bytes(saved))
    t.flags = flags
    ctx.check(ctx.lib.bg_set_tuning(ctx.h, C.byref(t)))
    try:
        return fn()
    finally:
        ctx.check(ctx.lib.bg_set_tuning(ctx.h, C.byref(saved)))


@pytest.mark.parametrize("w,h", [(48, 40), (37, 23)])
def test_tiled_pixel_order_changes_only_the_summation_order(gpu_ctx, w, h):
    """BG_TUNE_TILE_PIXELS hands the wavefront's camera rays out in 8 x 4 pixel tiles (ragged edges
    included): every pixel keeps its own samples, so the path and Whitted films equal the scanline
    order's up to the order of the film sums."""
    sd = S.env_sphere(w, h, spp=8, max_depth=5, extra=True)
    sc = G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)
    try:
        for it in (G.PathIntegrator(sd.camera, 8, 5), G.WhittedIntegrator(sd.camera, 8, 5)):
            a = _with_flags(gpu_ctx, 0, lambda: it.render(sc).rgb)
            b = _with_flags(gpu_ctx, A.BG_TUNE_TILE_PIXELS, lambda: it.render(sc).rgb)
            np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-6)
    finally:
        sc.close()


@pytest.mark.parametrize("mode,bvh,integrator", [(A.BG_MODE_PBRT, A.BG_BVH_WIDE, A.BG_INTEGRATOR_PATH),
                                                 (A.BG_MODE_REF_COMPAT, A.BG_BVH_REFERENCE_FIXED, A.BG_INTEGRATOR_PATH),
                                                 (A.BG_MODE_PBRT, A.BG_BVH_WIDE, A.BG_INTEGRATOR_WHITTED)])
@pytest.mark.parametrize("scene", ["example", "textured"])
def test_thin_lens_camera_matches_oracle(gpu_ctx, mode, bvh, integrator, scene):
    """PerspectiveCamera with a lens (perspective.rs:127-157): depth of field through the counter
    RNG's lens dimensions, and the ray differentials of a thin lens for texture filtering."""
    if scene == "example":
        sd = S.env_sphere(40, 32, spp=16, max_depth=5, extra=True)
        sd.camera.lens_radius, sd.camera.focal_distance = 0.3, 4.0
    else:
        sd = S.textured_room(40, 32, spp=16, max_depth=5)
        sd.camera.lens_radius, sd.camera.focal_distance = 0.15, 3.0
    o = O.OracleScene(sd, fixed_bvh=True).render(mode, spp=16, integrator=integrator)
    sc = G.Scene(gpu_ctx, sd, bvh)
    try:
        it = (G.PathIntegrator(sd.camera, 16, 5, mode=mode) if integrator == A.BG_INTEGRATOR_PATH
              else G.WhittedIntegrator(sd.camera, 16, 5, mode=mode))
        r = it.render(sc)
    finally:
        sc.close()
    s1, s2, n = G.PathIntegrator.moments(gpu_ctx, sd.camera.width, sd.camera.height)
    cmp = compare_renders(s1, s2, n, o["sum"], o["sumsq"], np.full(n.shape, 16))
    print(scene, cmp)
    assert r.stats.error_word == 0
    assert cmp["frac_z3"] <= 0.01
    assert cmp["frac_close"] >= 0.85


def test_camera_lens_arguments(gpu_ctx):
    sd = S.cornell(8, 8, spp=1)
    sc = G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)
    try:
        for lr, fd in ((-0.1, 1.0), (0.1, 0.0), (float("nan"), 1.0)):
            cam = S.Camera(sd.camera.position, sd.camera.look_at, sd.camera.up, sd.camera.fov_deg, 8, 8,
                           lens_radius=lr, focal_distance=fd)
            with pytest.raises(RuntimeError, match="lens|focal"):
                G.PathIntegrator(cam, 1, 2).render(sc)
    finally:
        sc.close()


def test_autotuner_picks_a_node_width(gpu_ctx, tmp_path, monkeypatch):
    """tune_layout builds the BVH 8-wide and 2-wide, keeps the faster, and the kept scene renders
    the same image as a scene built directly in that layout."""
    from bonsai_gb300 import autotune
    monkeypatch.setenv("BONSAI_TUNING_CACHE", str(tmp_path / "tuning.json"))
    sd = S.cornell(48, 48, spp=4)
    pi = G.PathIntegrator(sd.camera, 4, sd.max_depth, sd.rr_threshold, mode=A.BG_MODE_PBRT, seed=1)
    sc, info = autotune.tune_layout(gpu_ctx, sd, pi, spp=2)
    try:
        assert info["layout"] in autotune.LAYOUTS and len(info["trials"]) == 2 and not info["cached"]
        got = pi.render(sc).rgb
    finally:
        sc.close()
    ref_sc = G.Scene(gpu_ctx, sd, info["layout"])
    try:
        np.testing.assert_allclose(got, pi.render(ref_sc).rgb, rtol=1e-6, atol=1e-7)
    finally:
        ref_sc.close()
    sc2, info2 = autotune.tune_layout(gpu_ctx, sd, pi, spp=2)  # from the cache
    sc2.close()
    assert info2["cached"] and info2["layout"] == info["layout"]

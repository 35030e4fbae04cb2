"""DiffuseAreaLights on spheres, disks and cylinders (Shape::sample / pdf_from_it,
src/shapes/{sphere,disk,cylinder}.rs) on the device against the CPU oracle: the path, Whitted and
direct-lighting integrators in both estimator modes, with and without the Cornell box's triangle
light in the same light list."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from bonsai_gb300 import _abi as A
from bonsai_gb300 import gpu as G
from bonsai_gb300 import scenes as S

from .parity import compare_renders

pytestmark = pytest.mark.gpu

KINDS = [(A.BG_INTEGRATOR_PATH, 0), (A.BG_INTEGRATOR_WHITTED, 0), (A.BG_INTEGRATOR_DIRECT, A.BG_LIGHT_UNIFORM_ALL),
         (A.BG_INTEGRATOR_DIRECT, A.BG_LIGHT_UNIFORM_ONE)]


def _integrator(kind, strategy, cam, spp, depth, mode):
    if kind == A.BG_INTEGRATOR_PATH:
        return G.PathIntegrator(cam, spp, depth, mode=mode)
    if kind == A.BG_INTEGRATOR_WHITTED:
        return G.WhittedIntegrator(cam, spp, depth, mode=mode)
    return G.DirectLightingIntegrator(cam, spp, depth, strategy, mode=mode)


@pytest.mark.parametrize("kind,strategy", KINDS)
@pytest.mark.parametrize("mode,bvh", [(A.BG_MODE_PBRT, A.BG_BVH_WIDE), (A.BG_MODE_PBRT, A.BG_BVH_REFERENCE_FIXED),
                                      (A.BG_MODE_REF_COMPAT, A.BG_BVH_REFERENCE_FIXED)])
@pytest.mark.parametrize("tri_light", [True, False])
def test_shape_lights_match_oracle(gpu_ctx, kind, strategy, mode, bvh, tri_light):
    sd = S.shape_lights(40, 40, spp=16, max_depth=5, triangle_light=tri_light)
    o = O.OracleScene(sd, fixed_bvh=True).render(mode, spp=16, integrator=kind, light_strategy=strategy)
    sc = G.Scene(gpu_ctx, sd, bvh)
    try:
        r = _integrator(kind, strategy, sd.camera, 16, sd.max_depth, mode).render(sc)
    finally:
        sc.close()
    s1, s2, n = G.PathIntegrator.moments(gpu_ctx, sd.camera.width, sd.camera.height)
    cmp = compare_renders(s1, s2, n, o["sum"], o["sumsq"], np.full(n.shape, 16))
    print(kind, strategy, mode, cmp)
    assert r.stats.error_word == 0
    assert cmp["frac_z3"] <= 0.01
    assert cmp["frac_close"] >= 0.85
    assert r.rgb.mean() > 0.0


def test_shape_light_arguments(gpu_ctx):
    lib, ctx = gpu_ctx.lib, gpu_ctx
    h = C.c_void_p()
    ctx.check(lib.bg_scene_create(ctx.h, C.byref(h)))
    try:
        m = A.bg_material.from_buffer_copy(np.ascontiguousarray(S.material(S.MATTE)).tobytes())
        ctx.check(lib.bg_scene_add_material(h, C.byref(m), None))
        sph = np.zeros(1, S.SPHERE_DT)
        sph[0]["radius"], sph[0]["light_id"] = 0.5, 0  # no area light record yet
        assert lib.bg_scene_add_spheres(h, sph.ctypes.data, 1) == A.BG_ERR_INVALID
        l = A.bg_area_light()
        l.intensity[:] = (1.0, 1.0, 1.0)
        ctx.check(lib.bg_scene_add_area_light(h, C.byref(l), None))
        ctx.check(lib.bg_scene_add_spheres(h, sph.ctypes.data, 1))
        cone = S.quadric(S.CONE, np.eye(4), 0, radius=0.3, height=0.5)
        cone["light_id"] = 0
        qs = np.stack([cone])
        assert lib.bg_scene_add_quadrics(h, qs.ctypes.data, 1) == A.BG_ERR_UNSUPPORTED
        assert b"Cone" in lib.bg_last_error(ctx.h)
    finally:
        lib.bg_scene_destroy(h)


def test_emitting_shapes_in_batch_and_guided_renders(gpu_ctx):
    """The batch and guided paths share the shade code: an emitting-shape scene renders there to
    the same mean as a plain render."""
    sd = S.shape_lights(32, 32, spp=64, max_depth=5, triangle_light=False)
    sc = G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)
    try:
        plain = G.PathIntegrator(sd.camera, 64, 5, seed=2).render(sc).rgb
        imgs, st = G.render_batch(gpu_ctx, [G.BatchJob(sc, sd.camera, 64, 5, seed=2)])
        np.testing.assert_allclose(imgs[0], plain, rtol=1e-5, atol=1e-6)
        g = G.Guide(gpu_ctx, batch_size=4096, samples_per_pass=16384, warmup_passes=4, no_fallback=True,
                    pass_paths=32 * 32)
        try:
            gr = G.PathIntegrator(sd.camera, 64, 5, seed=9).render_guided(sc, g, spp=64)
            assert gr.stats.nan_samples == 0 and gr.stats.error_word == 0
            np.testing.assert_allclose(gr.rgb.mean(), plain.mean(), rtol=0.05)
        finally:
            g.close()
    finally:
        sc.close()

"""Edge cases of the render path through the C ABI: empty scenes, scenes without lights, depth 0,
a 1x1 film, spheres only, and rejected arguments (no fault, a status and a message)."""
import ctypes as C

import numpy as np
import pytest

from bonsai_gb300 import _abi as A
from bonsai_gb300 import gpu as G
from bonsai_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _empty_scene(ctx, kind=A.BG_BVH_WIDE, material=True):
    h = C.c_void_p()
    ctx.check(ctx.lib.bg_scene_create(ctx.h, C.byref(h)))
    if material:
        m = A.bg_material()
        m.type = A.BG_MAT_MATTE
        m.kd[:] = (0.5, 0.5, 0.5)
        ctx.check(ctx.lib.bg_scene_add_material(h, C.byref(m), None))
    st = A.bg_build_stats()
    ctx.check(ctx.lib.bg_scene_commit(h, kind, C.byref(st)))
    return h


def _render(ctx, h, cam, spp=2, depth=5, mode=A.BG_MODE_PBRT, flags=0):
    c = G.camera_struct(cam)
    o = A.bg_render_opts()
    o.spp, o.max_depth, o.rr_threshold, o.mode, o.seed, o.flags = spp, depth, 1.0, mode, 0, flags
    rgb = np.zeros((cam.height, cam.width, 3), np.float32)
    st = A.bg_render_stats()
    status = ctx.lib.bg_render(ctx.h, h, C.byref(c), C.byref(o), rgb.ctypes.data, C.byref(st))
    return status, rgb, st


@pytest.mark.parametrize("kind", [A.BG_BVH_WIDE, A.BG_BVH_WIDE2, A.BG_BVH_REFERENCE_FIXED])
def test_empty_scene_renders_black(gpu_ctx, kind):
    h = _empty_scene(gpu_ctx, kind)
    try:
        cam = S.cornell(16, 12).camera
        status, rgb, st = _render(gpu_ctx, h, cam)
        assert status == A.BG_OK and st.error_word == 0
        assert not rgb.any()
        rays = S.random_rays(64, seed=3)
        out = np.zeros(64, S.HIT_DT)
        gpu_ctx.check(gpu_ctx.lib.bg_trace_closest(gpu_ctx.h, h, rays.ctypes.data, 64, out.ctypes.data))
        assert (out["prim"] < 0).all()
    finally:
        gpu_ctx.lib.bg_scene_destroy(h)


def test_scene_without_lights_is_black(gpu_ctx):
    sd = S.cornell(24, 24, spp=4)
    keep = sd.tri_light < 0
    sd2 = S.SceneData(sd.tri[keep], sd.tri_mat[keep], sd.tri_light[keep], sd.spheres, sd.materials,
                      sd.lights[:0], sd.camera, spp=4, max_depth=5, rr_threshold=1.0)
    sc = G.Scene(gpu_ctx, sd2, A.BG_BVH_WIDE)
    try:
        r = G.PathIntegrator(sd.camera, 4, 5, mode=A.BG_MODE_PBRT).render(sc)
        assert r.stats.error_word == 0 and not r.rgb.any()
    finally:
        sc.close()


def test_depth_zero_sees_only_emission(gpu_ctx):
    sd = S.cornell(32, 32, spp=2)
    sc = G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)
    try:
        r = G.PathIntegrator(sd.camera, 2, 0, mode=A.BG_MODE_PBRT).render(sc)
        lit = r.rgb.sum(axis=2) > 0
        assert 0 < lit.mean() < 0.2  # the light quad only
        np.testing.assert_allclose(r.rgb[lit].max(axis=0), sd.lights[0]["intensity"], rtol=1e-5)
    finally:
        sc.close()


def test_one_pixel_film(gpu_ctx):
    sd = S.cornell(1, 1, spp=64)
    sc = G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)
    try:
        r = G.PathIntegrator(sd.camera, 64, 5, mode=A.BG_MODE_PBRT).render(sc)
        assert r.rgb.shape == (1, 1, 3) and np.isfinite(r.rgb).all() and r.stats.samples == 64
        _, _, n = G.PathIntegrator.moments(gpu_ctx, 1, 1)
        assert n[0, 0] == 64
    finally:
        sc.close()


def test_spheres_only_scene(gpu_ctx):
    sd = S.cornell(24, 24, spp=4)
    sd2 = S.SceneData(sd.tri[:0], sd.tri_mat[:0], sd.tri_light[:0], sd.spheres, sd.materials, sd.lights[:0],
                      sd.camera, spp=4, max_depth=3, rr_threshold=1.0)
    sc = G.Scene(gpu_ctx, sd2, A.BG_BVH_WIDE)
    try:
        rays = S.random_rays(4096, seed=5)
        rays["org"][:] = (0.0, -0.7, 2.0)  # in front of both spheres
        hits = sc.trace(rays)
        # spheres are numbered after the (zero) triangles: 0 and 1
        assert set(np.unique(hits["prim"])) <= {-1, 0, 1}
        assert (hits["prim"] == 0).any() and (hits["prim"] == 1).any() and (hits["prim"] < 0).any()
        assert np.isfinite(hits["t"][hits["prim"] >= 0]).all()
        r = G.PathIntegrator(sd.camera, 4, 3, mode=A.BG_MODE_PBRT).render(sc)
        assert r.stats.error_word == 0 and not r.rgb.any()  # no lights
    finally:
        sc.close()


def test_rejected_arguments(gpu_ctx):
    sd = S.cornell(8, 8, spp=1)
    sc = G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)
    try:
        cam = sd.camera
        assert _render(gpu_ctx, sc.h, cam, mode=7)[0] == A.BG_ERR_INVALID
        assert _render(gpu_ctx, sc.h, cam, depth=1000)[0] == A.BG_ERR_INVALID
        # REF_COMPAT needs a reference-layout BVH
        assert _render(gpu_ctx, sc.h, cam, mode=A.BG_MODE_REF_COMPAT)[0] == A.BG_ERR_INVALID
        assert b"REF_COMPAT" in gpu_ctx.lib.bg_last_error(gpu_ctx.h)
        bad = S.Camera(cam.position, cam.look_at, cam.up, 0.0, 8, 8)
        assert _render(gpu_ctx, sc.h, bad)[0] == A.BG_ERR_INVALID
        zero = S.Camera(cam.position, cam.look_at, cam.up, 40.0, 0, 8)
        assert _render(gpu_ctx, sc.h, zero)[0] == A.BG_ERR_INVALID
        # the context still renders afterwards
        status, rgb, st = _render(gpu_ctx, sc.h, cam)
        assert status == A.BG_OK and rgb.any()
    finally:
        sc.close()


def test_scene_builder_rejects_bad_records(gpu_ctx):
    lib, ctx = gpu_ctx.lib, gpu_ctx
    h = C.c_void_p()
    ctx.check(lib.bg_scene_create(ctx.h, C.byref(h)))
    try:
        tri = np.zeros((1, 9), np.float32)
        tri[0, 3] = np.nan
        mat = np.zeros(1, np.uint32)
        assert lib.bg_scene_add_triangles(h, tri.ctypes.data, 1, mat.ctypes.data, None) == A.BG_ERR_INVALID  # no material
        m = A.bg_material()
        m.type = 9
        assert lib.bg_scene_add_material(h, C.byref(m), None) == A.BG_ERR_INVALID
        m.type = A.BG_MAT_MATTE
        ctx.check(lib.bg_scene_add_material(h, C.byref(m), None))
        assert lib.bg_scene_add_triangles(h, tri.ctypes.data, 1, mat.ctypes.data, None) == A.BG_ERR_INVALID  # NaN
        sp = np.zeros(1, S.SPHERE_DT)
        sp["radius"] = -1.0
        sp["light_id"] = -1
        assert lib.bg_scene_add_spheres(h, sp.ctypes.data, 1) == A.BG_ERR_INVALID
        assert lib.bg_scene_commit(h, 77, None) == A.BG_ERR_INVALID
    finally:
        lib.bg_scene_destroy(h)

"""The InfiniteAreaLight (src/lights/infinite.rs) on the device against the CPU oracle: the
reference's example scene (src/main.rs: a UV-textured unit sphere under an environment map, camera
at (5, 0, 0)) and a variant whose light list mixes emitting triangles with the infinite light, for
the path, Whitted and direct-lighting integrators, in both estimator modes, over the BVH layouts."""
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
KINDS = [("path", A.BG_INTEGRATOR_PATH, 0), ("whitted", A.BG_INTEGRATOR_WHITTED, 0),
         ("direct_all", A.BG_INTEGRATOR_DIRECT, A.BG_LIGHT_UNIFORM_ALL),
         ("direct_one", A.BG_INTEGRATOR_DIRECT, A.BG_LIGHT_UNIFORM_ONE)]


def _integrator(kind, strategy, cam, spp, depth, mode):
    if kind == A.BG_INTEGRATOR_PATH:
        return G.PathIntegrator(cam, spp, depth, mode=mode)
    if kind == A.BG_INTEGRATOR_WHITTED:
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


@pytest.mark.parametrize("bvh", [A.BG_BVH_WIDE, A.BG_BVH_WIDE2, A.BG_BVH_REFERENCE_FIXED])
def test_reference_example_scene_pbrt(gpu_ctx, bvh):
    sd = S.env_sphere(48, 48, spp=16, max_depth=5)
    r, o, cmp = _pair(gpu_ctx, sd, A.BG_INTEGRATOR_PATH, 0, A.BG_MODE_PBRT, bvh, 16)
    print(cmp)
    assert r.stats.error_word == 0
    assert cmp["frac_z3"] <= Z3_FRAC
    assert cmp["frac_close"] >= 0.9
    np.testing.assert_allclose(r.rgb.mean(), o["rgb"].mean(), rtol=2e-3)


def test_reference_example_scene_ref_compat(gpu_ctx):
    sd = S.env_sphere(48, 48, spp=16, max_depth=5)
    r, o, cmp = _pair(gpu_ctx, sd, A.BG_INTEGRATOR_PATH, 0, A.BG_MODE_REF_COMPAT, A.BG_BVH_REFERENCE_FIXED, 16)
    print(cmp)
    assert cmp["frac_z3"] <= Z3_FRAC
    assert cmp["frac_close"] >= 0.9


@pytest.mark.parametrize("name,kind,strategy", KINDS)
@pytest.mark.parametrize("bvh", [A.BG_BVH_WIDE, A.BG_BVH_REFERENCE_FIXED])
def test_mixed_lights_pbrt(gpu_ctx, name, kind, strategy, bvh):
    """Two emitting triangles and the infinite light share the light list; glass and plastic
    spheres give specular chains that escape to the environment."""
    sd = S.env_sphere(40, 40, spp=16, max_depth=5, extra=True)
    r, o, cmp = _pair(gpu_ctx, sd, kind, strategy, A.BG_MODE_PBRT, bvh, 16)
    print(name, cmp)
    assert r.stats.error_word == 0
    assert cmp["frac_z3"] <= Z3_FRAC
    assert cmp["frac_close"] >= 0.85


@pytest.mark.parametrize("name,kind,strategy", KINDS)
def test_mixed_lights_ref_compat(gpu_ctx, name, kind, strategy):
    sd = S.env_sphere(40, 40, spp=16, max_depth=5, extra=True)
    r, o, cmp = _pair(gpu_ctx, sd, kind, strategy, A.BG_MODE_REF_COMPAT, A.BG_BVH_REFERENCE_FIXED, 16)
    print(name, cmp)
    assert cmp["frac_z3"] <= Z3_FRAC
    assert cmp["frac_close"] >= 0.85


def test_uniform_environment_furnace(gpu_ctx):
    """A grey sphere (albedo 0.5) under a uniform unit environment renders 0.5 (PBRT); pixels that
    miss it show the map, 1."""
    sd = S.env_sphere(32, 32, spp=256, max_depth=1)
    sd.env.rgb = np.ones((16, 32, 3), np.float32)
    sd.materials = np.stack([S.material(S.MATTE, kd=(0.5, 0.5, 0.5))])
    sd.textures = []
    sc = G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)
    try:
        rgb = G.PathIntegrator(sd.camera, 256, 1).render(sc).rgb
    finally:
        sc.close()
    np.testing.assert_allclose(rgb[14:18, 14:18].mean(), 0.5, atol=0.01)
    np.testing.assert_allclose(rgb[0, 0], 1.0, atol=1e-5)


def test_noalloc_renders_the_environment(gpu_ctx):
    sd = S.env_sphere(32, 24, spp=4, extra=True)
    scene = G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)
    try:
        cam = G.camera_struct(sd.camera)
        o = A.bg_render_opts()
        o.spp, o.max_depth, o.rr_threshold, o.mode, o.seed = 4, 5, 1.0, A.BG_MODE_PBRT, 3
        want = np.zeros((24, 32, 3), np.float32)
        st = A.bg_render_stats()
        gpu_ctx.check(gpu_ctx.lib.bg_render(gpu_ctx.h, scene.h, C.byref(cam), C.byref(o), want.ctypes.data,
                                            C.byref(st)))
        d_out = gpu_ctx.alloc(want.nbytes)
        try:
            gpu_ctx.check(gpu_ctx.lib.bg_render_noalloc(scene.h, C.byref(cam), C.byref(o), d_out, None))
            got = np.zeros_like(want)
            gpu_ctx.d2h(got, d_out)
        finally:
            gpu_ctx.free(d_out)
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)
        assert want[0, 0].sum() > 0.0
    finally:
        scene.close()


def test_infinite_light_arguments(gpu_ctx):
    lib, ctx = gpu_ctx.lib, gpu_ctx
    h = C.c_void_p()
    ctx.check(lib.bg_scene_create(ctx.h, C.byref(h)))
    try:
        npot = S.EnvMap(np.ones((12, 24, 3), np.float32))
        el, keep = S.env_struct(npot)
        assert lib.bg_scene_add_infinite_light(h, C.byref(el)) == A.BG_ERR_UNSUPPORTED
        assert b"powers of two" in lib.bg_last_error(ctx.h)
        sing = S.EnvMap(np.ones((8, 16, 3), np.float32), light_to_world=np.zeros((3, 4), np.float32))
        el, keep = S.env_struct(sing)
        assert lib.bg_scene_add_infinite_light(h, C.byref(el)) == A.BG_ERR_INVALID
        bad = np.ones((8, 16, 3), np.float32)
        bad[3, 4, 1] = -0.5
        el, keep = S.env_struct(S.EnvMap(bad))
        assert lib.bg_scene_add_infinite_light(h, C.byref(el)) == A.BG_ERR_INVALID
        bad[3, 4, 1] = np.inf
        el, keep = S.env_struct(S.EnvMap(bad))
        assert lib.bg_scene_add_infinite_light(h, C.byref(el)) == A.BG_ERR_INVALID
        ok = S.EnvMap(np.ones((8, 16, 3), np.float32))
        el, keep = S.env_struct(ok)
        ctx.check(lib.bg_scene_add_infinite_light(h, C.byref(el)))
        assert lib.bg_scene_add_infinite_light(h, C.byref(el)) == A.BG_ERR_UNSUPPORTED
        assert lib.bg_scene_add_infinite_light(h, None) == A.BG_ERR_INVALID
    finally:
        lib.bg_scene_destroy(h)


@pytest.mark.parametrize("mode,bvh", [(A.BG_MODE_PBRT, A.BG_BVH_WIDE),
                                      (A.BG_MODE_REF_COMPAT, A.BG_BVH_REFERENCE_FIXED)])
def test_rotated_and_tinted_environment(gpu_ctx, mode, bvh):
    """A light_to_world rotation (the map's pole tilted 35 degrees about x, then turned 70 degrees
    about z) and a per-channel intensity, against the oracle."""
    sd = S.env_sphere(40, 40, spp=16, max_depth=4, extra=True, seed=5)
    rot = S.rotation((0, 0, 1), 70.0) @ S.rotation((1, 0, 0), 35.0)
    sd.env.light_to_world = rot[:3].astype(np.float32)
    sd.env.intensity = (1.5, 1.0, 0.6)
    r, o, cmp = _pair(gpu_ctx, sd, A.BG_INTEGRATOR_PATH, 0, mode, bvh, 16)
    print(cmp)
    assert cmp["frac_z3"] <= Z3_FRAC
    assert cmp["frac_close"] >= 0.85


def test_environment_map_shapes(gpu_ctx):
    """Degenerate maps: 1 x 1 (a single level, a 2 x 2 distribution), 1 x 64 and 64 x 1."""
    for h, w in ((1, 1), (1, 64), (64, 1), (2, 4)):
        sd = S.env_sphere(24, 24, spp=8, max_depth=3)
        rng = np.random.default_rng(h * 100 + w)
        sd.env.rgb = (0.2 + rng.random((h, w, 3))).astype(np.float32)
        r, o, cmp = _pair(gpu_ctx, sd, A.BG_INTEGRATOR_PATH, 0, A.BG_MODE_PBRT, A.BG_BVH_WIDE, 8)
        assert cmp["frac_z3"] <= Z3_FRAC, (h, w, cmp)
        assert cmp["frac_close"] >= 0.85, (h, w, cmp)

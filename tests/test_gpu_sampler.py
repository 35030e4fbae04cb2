"""The StratifiedSampler (src/samplers/stratified.rs) on the device against the CPU oracle: the path
integrator's wavefront (PBRT) and per-sample kernel (both modes), CUDA-graph replay, the
allocation-free entry point, Whitted's camera-only stratification, and the argument checks."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from bonsai_gb300 import _abi as A
from bonsai_gb300 import gpu as G
from bonsai_gb300 import scenes as S

from .parity import compare_renders

pytestmark = pytest.mark.gpu

MAIN = S.StratifiedSampler(4, 4, 4, True)  # the reference's example sampler


def _pair(ctx, sd, mode, bvh, sampler, integrator=A.BG_INTEGRATOR_PATH, first_sample=0):
    spp = sampler.spp
    o = O.OracleScene(sd, fixed_bvh=True).render(mode, spp=spp, sampler=sampler, integrator=integrator,
                                                 first_sample=first_sample)
    sc = G.Scene(ctx, sd, bvh)
    try:
        if integrator == A.BG_INTEGRATOR_PATH:
            it = G.PathIntegrator(sd.camera, spp, sd.max_depth, sd.rr_threshold, mode=mode, sampler=sampler)
        else:
            it = G.WhittedIntegrator(sd.camera, spp, sd.max_depth, mode=mode, sampler=sampler)
        r = it.render(sc, first_sample=first_sample)
    finally:
        sc.close()
    s1, s2, n = G.PathIntegrator.moments(ctx, sd.camera.width, sd.camera.height)
    return r, o, compare_renders(s1, s2, n, o["sum"], o["sumsq"], np.full(n.shape, spp))


@pytest.mark.parametrize("mode,bvh", [(A.BG_MODE_PBRT, A.BG_BVH_WIDE), (A.BG_MODE_PBRT, A.BG_BVH_REFERENCE_FIXED),
                                      (A.BG_MODE_REF_COMPAT, A.BG_BVH_REFERENCE_FIXED)])
@pytest.mark.parametrize("scene", ["example", "cornell", "textured"])
def test_stratified_path_matches_oracle(gpu_ctx, mode, bvh, scene):
    """"textured": image textures filtered with the camera ray's differentials at the stratified
    film position."""
    if scene == "example":
        sd = S.env_sphere(40, 40, spp=16, max_depth=5, extra=True)
    elif scene == "cornell":
        sd = S.cornell(40, 40, 16, 6)
    else:
        sd = S.textured_room(40, 40, spp=16, max_depth=5)
    r, o, cmp = _pair(gpu_ctx, sd, mode, bvh, MAIN)
    print(scene, cmp)
    assert r.stats.error_word == 0
    assert cmp["frac_z3"] <= 0.01
    assert cmp["frac_close"] >= 0.9


def test_stratified_later_pass_and_all_dimensions(gpu_ctx):
    """A second pass (first_sample = spp) and every call stratified (sampled_dimensions 64 covers a
    depth-8 path), 3 x 2 grid without jitter."""
    sd = S.cornell(32, 32, 6, 8)
    r, o, cmp = _pair(gpu_ctx, sd, A.BG_MODE_PBRT, A.BG_BVH_WIDE, S.StratifiedSampler(3, 2, 64, False),
                      first_sample=6)
    assert cmp["frac_z3"] <= 0.01 and cmp["frac_close"] >= 0.9, cmp


def test_graph_replay_matches_direct_launches(gpu_ctx):
    sd = S.env_sphere(32, 32, spp=16, max_depth=5)
    sc = G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)
    try:
        it = G.PathIntegrator(sd.camera, 16, 5, sampler=MAIN)
        out = []
        for graph in (False, True, True):
            out.append(it.render(sc, first_sample=16 * len(out), graph=graph).rgb)
        plain = it.render(sc, first_sample=32, graph=False).rgb
    finally:
        sc.close()
    np.testing.assert_allclose(out[2], plain, rtol=1e-6, atol=1e-7)


def test_noalloc_takes_the_stratified_sampler(gpu_ctx):
    sd = S.env_sphere(32, 24, spp=16, extra=True)
    scene = G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)
    try:
        cam = G.camera_struct(sd.camera)
        o = A.bg_render_opts()
        o.spp, o.max_depth, o.rr_threshold, o.mode, o.seed = 16, 5, 1.0, A.BG_MODE_PBRT, 3
        S.set_sampler(o, MAIN)
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
    finally:
        scene.close()


@pytest.mark.parametrize("mode,bvh", [(A.BG_MODE_PBRT, A.BG_BVH_WIDE), (A.BG_MODE_REF_COMPAT, A.BG_BVH_REFERENCE_FIXED)])
def test_whitted_stratifies_the_camera_sample(gpu_ctx, mode, bvh):
    sd = S.env_sphere(32, 32, spp=16, max_depth=4, extra=True)
    r, o, cmp = _pair(gpu_ctx, sd, mode, bvh, S.StratifiedSampler(4, 4, 1, True), integrator=A.BG_INTEGRATOR_WHITTED)
    assert cmp["frac_z3"] <= 0.01 and cmp["frac_close"] >= 0.9, cmp


def test_sampler_arguments(gpu_ctx):
    sd = S.cornell(8, 8, spp=4)
    sc = G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)
    try:
        with pytest.raises(RuntimeError, match="x_pixel_samples"):
            G.PathIntegrator(sd.camera, 4, 3, sampler=S.StratifiedSampler(3, 2, 1)).render(sc)
        with pytest.raises(RuntimeError, match="sampled_dimensions"):
            G.PathIntegrator(sd.camera, 4, 3, sampler=S.StratifiedSampler(2, 2, 65)).render(sc)
        with pytest.raises(RuntimeError, match="sampled_dimensions <= 1"):
            G.WhittedIntegrator(sd.camera, 4, 3, sampler=S.StratifiedSampler(2, 2, 2)).render(sc)
        it = G.PathIntegrator(sd.camera, 4, 3)
        it.sampler = S.StratifiedSampler(2, 2, 1)
        with pytest.raises(RuntimeError, match="x_pixel_samples"):  # batch items are checked alike
            G.render_batch(gpu_ctx, [G.BatchJob(sc, sd.camera, 4, 3, sampler=S.StratifiedSampler(4, 2, 1))])
    finally:
        sc.close()


def test_stratified_lens_samples(gpu_ctx):
    """sampled_dimensions >= 2: the thin lens takes the sampler's second get_2d call."""
    sd = S.env_sphere(40, 32, spp=16, max_depth=5, extra=True)
    sd.camera.lens_radius, sd.camera.focal_distance = 0.3, 4.0
    r, o, cmp = _pair(gpu_ctx, sd, A.BG_MODE_PBRT, A.BG_BVH_WIDE, MAIN)
    assert cmp["frac_z3"] <= 0.01 and cmp["frac_close"] >= 0.85, cmp

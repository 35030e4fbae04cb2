"""Uneven multi-scene batch (bg_render_batch): every scene's film equals its own single-scene
render (same counter RNG, same estimator, same paths), with waves small enough that paths of
different scenes share a wave.  The batch's shade kernels are separate instances of the shading
code (per-path scenes), compiled, like the single-scene ones, with fused multiply-adds: where the
compiler contracts an expression differently in the two instances the results differ in the last
bits, so films agree to 1e-4 relative (and the FP64 moments likewise), not bit for bit
(tests.parity.assert_same_paths)."""
import numpy as np
import pytest

from bonsai_gb300 import _abi as A
from bonsai_gb300 import autotune
from bonsai_gb300 import gpu as G
from bonsai_gb300 import scenes as S

from .parity import assert_same_paths

pytestmark = pytest.mark.gpu


def _moments_flat(ctx, npix):
    return G.PathIntegrator.moments(ctx, npix, 1)


@pytest.mark.parametrize("wave_paths", [1 << 16, 1 << 22])
def test_batch_matches_single_scene_renders(gpu_ctx, wave_paths):
    sds = S.uneven_batch(6, seed=11, max_tris=30_000)
    for sd in sds:
        sd.spp = min(sd.spp, 6)
    scenes = [G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE) for sd in sds]
    old = autotune.get(gpu_ctx)
    try:
        autotune.set_(gpu_ctx, old.refill, old.blocks_per_sm, wave_paths)
        jobs = [G.BatchJob(sc, sd.camera, sd.spp, sd.max_depth, seed=3) for sc, sd in zip(scenes, sds)]
        imgs, st = G.render_batch(gpu_ctx, jobs)
        npix = [sd.camera.width * sd.camera.height for sd in sds]
        assert st.samples == sum(n * sd.spp for n, sd in zip(npix, sds))
        assert st.error_word == 0 and st.nan_samples == 0
        b1, b2, bn = _moments_flat(gpu_ctx, sum(npix))
        off = 0
        for sc, sd, img, n in zip(scenes, sds, imgs, npix):
            pi = G.PathIntegrator(sd.camera, sd.spp, sd.max_depth, mode=A.BG_MODE_PBRT, seed=3)
            r = pi.render(sc)
            s1, s2, cnt = G.PathIntegrator.moments(gpu_ctx, sd.camera.width, sd.camera.height)
            np.testing.assert_array_equal(bn[0, off:off + n], cnt.reshape(-1))
            assert_same_paths(b1[0, off:off + n], s1.reshape(-1, 3))
            assert_same_paths(b2[0, off:off + n], s2.reshape(-1, 3), rtol=2e-4)
            assert_same_paths(img, r.rgb)
            off += n
    finally:
        autotune.set_(gpu_ctx, old.refill, old.blocks_per_sm, old.wave_paths)
        for sc in scenes:
            sc.close()


def test_batch_rejects_non_wide_scenes(gpu_ctx):
    sd = S.cornell(32, 32, spp=2)
    sc = G.Scene(gpu_ctx, sd, A.BG_BVH_REFERENCE_FIXED)
    try:
        with pytest.raises(G.BonsaiError):
            G.render_batch(gpu_ctx, [G.BatchJob(sc, sd.camera, 2, 3)])
    finally:
        sc.close()


def test_batch_mixes_textures_infinite_lights_and_samplers(gpu_ctx):
    """A batch of the reference's example scene (UV texture, infinite light, two emitting triangles;
    4x4 stratified sampler), the textured room (image textures filtered with ray differentials)
    and the Cornell box (independent sampler): each film equals its single-scene render."""
    sds = [S.env_sphere(40, 32, spp=16, max_depth=5, extra=True), S.textured_room(24, 24, spp=4, max_depth=5),
           S.cornell(16, 24, spp=4, max_depth=4)]
    samplers = [S.StratifiedSampler(4, 4, 4, True), S.StratifiedSampler(2, 2, 2, False), None]
    scenes = [G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE) for sd in sds]
    try:
        jobs = [G.BatchJob(sc, sd.camera, sd.spp, sd.max_depth, seed=5, sampler=smp)
                for sc, sd, smp in zip(scenes, sds, samplers)]
        imgs, st = G.render_batch(gpu_ctx, jobs)
        assert st.error_word == 0
        for sc, sd, smp, img in zip(scenes, sds, samplers, imgs):
            r = G.PathIntegrator(sd.camera, sd.spp, sd.max_depth, seed=5, sampler=smp).render(sc)
            assert_same_paths(img, r.rgb)
            assert img.mean() > 0.0
    finally:
        for sc in scenes:
            sc.close()

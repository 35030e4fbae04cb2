"""Failure paths of the library, made on the host; none of them faults or hangs the GPU.

The reference only panics (`expect`/`unwrap`, e.g. src/base/bsdf.rs:162); at the C ABI every
failure is a bg_status with a message, and the context stays usable afterwards:
  * a device memory cap smaller than the scene        -> BG_ERR_OOM, before any cudaMalloc;
  * a shadow-ray queue too small for a bounce          -> BG_ERR_DEVICE (queue overflow): the
    shade kernel's bounds check drops the excess rays and records the error word;
  * a tensor-core wait of the guiding network that runs out of its (deliberately short) limit
    -> BG_ERR_TIMEOUT: the kernels let the issued MMAs retire, free TMEM and return.
Each test then renders (or runs the network) again on the same context and checks the result.
"""
import ctypes as C

import numpy as np
import pytest

from bonsai_gb300 import _abi as A
from bonsai_gb300 import autotune
from bonsai_gb300 import gpu as G
from bonsai_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _render(ctx, sd, seed=0):
    sc = G.Scene(ctx, sd, A.BG_BVH_WIDE)
    try:
        return G.PathIntegrator(sd.camera, sd.spp, sd.max_depth, sd.rr_threshold, mode=A.BG_MODE_PBRT,
                                seed=seed).render(sc).rgb
    finally:
        sc.close()


def test_memory_cap_gives_oom_and_context_stays_usable(gpu_ctx):
    small = S.cornell(24, 24, spp=2)
    want = _render(gpu_ctx, small)
    ctx = G.Context(0, memory_cap_bytes=8 << 20)
    try:
        big, _ = S.ray_soup(400_000, 16)  # 19.2 MB of triangles alone
        with pytest.raises(G.BonsaiError) as ei:
            G.Scene(ctx, big, A.BG_BVH_WIDE)
        assert ei.value.status == A.BG_ERR_OOM
        assert "cap" in str(ei.value)
        got = _render(ctx, small)  # the same context, within the cap
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)
    finally:
        ctx.close()


def _lit_floor(w=32, h=32, spp=4):
    """A matte floor under a two-sided area light 0.2 above it, both 100 x 100, seen by a camera
    between the two: from every floor point nearly every BSDF sample reaches the light, so nearly
    every vertex queues two shadow rays (the light sample and the MIS ray toward the light)."""
    floor = S._quad((-50, -1, -50), (50, -1, -50), (50, -1, 50), (-50, -1, 50), (0, 1, 0))
    light = S._quad((-50, -0.8, -50), (50, -0.8, -50), (50, -0.8, 50), (-50, -0.8, 50), (0, -1, 0))
    tri = np.concatenate([floor, light]).astype(np.float32)
    mats = np.stack([S.material(S.MATTE, kd=(0.5, 0.5, 0.5)), S.material(S.MATTE, kd=(0, 0, 0))])
    lights = np.zeros(1, S.LIGHT_DT)
    lights[0] = ((1.0, 1.0, 1.0), 1)
    cam = S.Camera((0.0, -0.9, 0.0), (0.0, -1.0, -0.05), (0.0, 1.0, 0.0), 60.0, w, h)  # every ray meets the floor
    return S.SceneData(tri, np.array([0, 0, 1, 1], np.uint32), np.array([-1, -1, 0, 0], np.int32),
                       np.zeros(0, S.SPHERE_DT), mats, lights, cam, spp=spp, max_depth=3, rr_threshold=1.0,
                       name="lit_floor")


def test_shadow_queue_overflow_is_reported(gpu_ctx):
    sd = _lit_floor()
    want = _render(gpu_ctx, sd)
    t0 = autotune.get(gpu_ctx)
    t = A.bg_tuning()
    t.wave_paths, t.blocks_per_sm, t.refill = t0.wave_paths, t0.blocks_per_sm, t0.refill
    t.flags = t0.flags | A.BG_TUNE_SHADOW_QUEUE_HALF
    gpu_ctx.check(gpu_ctx.lib.bg_set_tuning(gpu_ctx.h, C.byref(t)))
    try:
        with pytest.raises(G.BonsaiError) as ei:
            _render(gpu_ctx, sd)
        assert ei.value.status == A.BG_ERR_DEVICE
        assert "queue overflow" in str(ei.value)
    finally:
        gpu_ctx.check(gpu_ctx.lib.bg_set_tuning(gpu_ctx.h, C.byref(t0)))
    got = _render(gpu_ctx, sd)  # full queue again: the same image as before
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)


def test_guide_wait_timeout_then_recovery(gpu_ctx):
    from oracle import guide as OG
    g = G.Guide(gpu_ctx, batch_size=1024, samples_per_pass=4096)
    try:
        g.params = OG.init_params(3)
        q = OG.random_samples(2048, 4)[:, :9]
        want = g.forward(q)
        g.set_wait_limit(8)  # far below one MMA's latency: every launch gives up
        try:
            with pytest.raises(G.BonsaiError) as ei:
                g.forward(q)
            assert ei.value.status == A.BG_ERR_TIMEOUT
            s = OG.random_samples(1024, 5)
            with pytest.raises(G.BonsaiError) as ei:
                g.gradient(s)
            assert ei.value.status == A.BG_ERR_TIMEOUT
        finally:
            g.set_wait_limit(0)
        np.testing.assert_array_equal(g.forward(q), want)  # default limit: the same outputs
        grad, loss = g.gradient(OG.random_samples(1024, 5))
        assert np.isfinite(loss) and np.isfinite(grad).all()
    finally:
        g.close()

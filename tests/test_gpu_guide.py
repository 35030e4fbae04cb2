"""GPU parity of the guiding network (tcgen05 forward / backward / Adam) against the FP64 oracle,
of the mixture device functions, and of guided rendering (unbiased, and better than plain BSDF
sampling once trained).

Tolerances (stated here, measured values are printed with -s):
  forward   relative L2 error vs the BF16-emulating oracle < 2e-3 (FP32 accumulation order only),
            vs exact FP64 < 3e-2 (the BF16 operand error);
  gradient  relative L2 error vs the BF16-emulating oracle < 2e-2, vs exact FP64 < 8e-2;
            batch loss within 1e-2 (relative) of the FP64 loss;
  Adam      parameters within 2e-6 of the oracle's step applied to the GPU gradient.
"""
import numpy as np
import pytest

from bonsai_gb300 import _abi as A
from bonsai_gb300 import gpu as G
from bonsai_gb300 import scenes as S
from oracle import guide as O

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="module")
def guide(gpu_ctx):
    g = G.Guide(gpu_ctx, batch_size=1024, samples_per_pass=4096)
    yield g
    g.close()


def test_forward_matches_fp64(guide):
    p = O.init_params(1)
    guide.params = p
    q = O.random_samples(1000, 2)[:, :9]
    out = guide.forward(q)
    ref_bf = O.forward(p, q, bf16_sim=True)[0][:, :O.OUT]
    ref = O.forward(p, q)[0][:, :O.OUT]
    e_bf, e = _rel(out, ref_bf), _rel(out, ref)
    print(f"forward rel L2 error: vs BF16 oracle {e_bf:.2e}, vs FP64 {e:.2e}")
    assert e_bf < 2e-3
    assert e < 3e-2


@pytest.mark.parametrize("n", [1, 127, 128, 129, 300, 4097])
def test_forward_ragged_batches(guide, n):
    p = O.init_params(7)
    guide.params = p
    q = O.random_samples(n, 8)[:, :9]
    out = guide.forward(q)
    assert out.shape == (n, O.OUT) and np.isfinite(out).all()
    ref = O.forward(p, q, bf16_sim=True)[0][:, :O.OUT]
    assert _rel(out, ref) < 2e-3


def test_params_roundtrip_and_padding_check(guide):
    p = O.init_params(9)
    guide.params = p
    np.testing.assert_array_equal(guide.params, p)
    bad = p.copy()
    bad[O.param_off(1) + 3 * O.K + 70] = 1.0  # a padding column of layer 1
    with pytest.raises(G.BonsaiError):
        guide.params = bad
    guide.params = p


def test_gradient_matches_fp64(guide):
    p = O.init_params(3)
    guide.params = p
    s = O.random_samples(2048, 4)
    g, loss = guide.gradient(s)
    gb, lb = O.batch_loss_grad(p, s, bf16_sim=True)
    gr, lr = O.batch_loss_grad(p, s)
    e_bf, e = _rel(g, gb), _rel(g, gr)
    cos = float(np.dot(g, gr) / (np.linalg.norm(g) * np.linalg.norm(gr)))
    print(f"gradient rel L2 error: vs BF16 oracle {e_bf:.2e}, vs FP64 {e:.2e}, cosine {cos:.6f}; "
          f"loss {loss:.6f} vs FP64 {lr:.6f} (rel {abs(loss - lr) / abs(lr):.2e})")
    assert e_bf < 2e-2
    assert e < 8e-2
    assert abs(loss - lr) <= 1e-2 * abs(lr)
    # padding never receives gradient
    for l in range(O.LAYERS):
        W = g[O.param_off(l):O.param_off(l) + O.rows(l) * O.K].reshape(O.rows(l), O.K)
        assert not W[O.used_rows(l):].any()


def test_gradient_all_zero_weights(guide):
    guide.params = O.init_params(3)
    s = O.random_samples(256, 4)
    s[:, 13:15] = 0.0
    g, loss = guide.gradient(s)
    assert not g.any() and loss == 0.0


def test_adam_step_matches_oracle(gpu_ctx):
    g = G.Guide(gpu_ctx, batch_size=1024, samples_per_pass=4096, learning_rate=1e-3)
    try:
        p = O.init_params(5)
        g.params = p
        s = O.random_samples(1024, 6)
        grad, _ = g.gradient(s)
        g.train(s)
        p1 = g.params
        ref, _, _ = O.adam(p.astype(np.float64), 0.0, 0.0, grad.astype(np.float64), 1)
        assert np.abs(p1 - ref).max() < 2e-6
        assert np.array_equal(p1 == 0, p == 0) or np.abs(p1[p == 0]).max() < 2e-6
    finally:
        g.close()


def test_training_fits_a_known_distribution(gpu_ctx):
    """Samples drawn from a fixed two-lobe distribution with unit weights: the loss must fall
    towards the distribution's entropy and the learnt density must concentrate on the lobes."""
    g = G.Guide(gpu_ctx, batch_size=1024, samples_per_pass=1 << 14, learning_rate=3e-3)
    try:
        rng = np.random.default_rng(0)
        n = 1 << 14
        raw_t = np.zeros((n, O.HEAD_OUT))
        raw_t[:, 0:3] = (1.0, 0.0, 0.0)
        raw_t[:, 3] = np.log(20.0)
        raw_t[:, 5:8] = (0.0, 0.0, 1.0)
        raw_t[:, 8] = np.log(20.0)
        raw_t[:, 9] = 0.0
        raw_t[:, 14:40:5] = -30.0  # other lobes off
        raw_t[:, 4] = 0.0
        wi = O.sample(raw_t, rng.random((n, 3)))
        s = O.random_samples(n, 1)
        s[:, 9:12] = wi
        s[:, 12] = 0.0          # no BSDF: the mixture is the guide alone
        s[:, 13] = 1.0          # head 0 learns the two lobes, head 1 gets no samples
        s[:, 14] = 0.0
        losses = [g.train(s) for _ in range(40)]
        print("loss", losses[0], "->", losses[-1])
        assert losses[-1] < losses[0] - 1.0
        out = g.forward(s[:512, :9])
        on = O.pdf(out, np.tile([1.0, 0.0, 0.0], (512, 1))) + O.pdf(out, np.tile([0.0, 0.0, 1.0], (512, 1)))
        off = O.pdf(out, np.tile([-1.0, 0.0, 0.0], (512, 1)))  # head 0 (the first 41 outputs)
        assert np.median(on) > 10 * np.median(off)
    finally:
        g.close()


def test_mixture_eval_matches_oracle(guide):
    rng = np.random.default_rng(21)
    n = 4096
    raw = rng.normal(0, 1, (n, O.HEAD_OUT))
    raw[:, 3:40:5] = rng.uniform(-2.5, 8.5, (n, O.LOBES))  # includes clamped log kappa
    u = rng.random((n, 3))
    w = rng.normal(size=(n, 3))
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    pb = np.where(rng.random(n) < 0.2, 0.0, rng.exponential(0.5, n))
    raw32, u32, w32, pb32 = (a.astype(np.float32) for a in (raw, u, w, pb))
    out = guide.mixture_eval(raw32, u32, w32, pb32)
    r64, u64, w64, p64 = (a.astype(np.float64) for a in (raw32, u32, w32, pb32))
    ws = O.sample(r64, u64)
    close = np.linalg.norm(out[:, :3] - ws, axis=1) < 1e-3
    assert close.mean() > 0.995  # lobe picks at a CDF boundary may differ between FP32 and FP64
    np.testing.assert_allclose(out[close, 3], O.pdf(r64[close], ws[close]), rtol=5e-3, atol=1e-6)
    np.testing.assert_allclose(out[:, 4], O.pdf(r64, w64), rtol=5e-3, atol=1e-6)
    m = O.parse(r64)
    np.testing.assert_allclose(out[:, 5], m["c"], rtol=1e-5)
    loss, g = O.loss_grad(r64, w64, p64, np.ones(n))
    np.testing.assert_allclose(out[:, 6], loss, rtol=2e-3, atol=1e-4)
    np.testing.assert_allclose(out[:, 8:48], g[:, :40], rtol=5e-3, atol=5e-4 * np.abs(g[:, :40]).max())
    np.testing.assert_allclose(out[:, 7], g[:, 40], rtol=5e-3, atol=1e-5)


# ---------------------------------------------------------------- guided rendering
def _small_slit(w=96, h=64, depth=6):
    return S.slit_room(w, h, n_ico=2, ico_level=2, n_spheres=20, max_depth=depth, light_intensity=200.0)


def _block_z(s1a, s2a, na, s1b, s2b, nb, bs=8):
    """z-scores of 8x8-block means of two independent renders (per-pixel sample variances)."""
    def stats(s1, s2, n):
        n = n[..., None].astype(np.float64)
        m = s1 / n
        var = np.maximum(s2 / n - m * m, 0.0) / n
        H, W = m.shape[:2]
        mb = m[:H // bs * bs, :W // bs * bs].reshape(H // bs, bs, W // bs, bs, 3).mean(axis=(1, 3))
        vb = var[:H // bs * bs, :W // bs * bs].reshape(H // bs, bs, W // bs, bs, 3).sum(axis=(1, 3)) / bs ** 4
        return mb, vb
    ma, va = stats(s1a, s2a, na)
    mb, vb = stats(s1b, s2b, nb)
    return (ma - mb) / np.sqrt(va + vb + 1e-30)


def test_guided_render_is_unbiased(gpu_ctx):
    sd = _small_slit()
    sc = G.Scene(gpu_ctx, sd)
    npix = sd.camera.width * sd.camera.height
    g = G.Guide(gpu_ctx, batch_size=4096, samples_per_pass=16384, warmup_passes=4, no_fallback=True, pass_paths=npix)
    try:
        pi = G.PathIntegrator(sd.camera, 512, sd.max_depth, mode=A.BG_MODE_PBRT, seed=5)
        pi.render(sc, spp=512)
        p1, p2, pn = G.PathIntegrator.moments(gpu_ctx, sd.camera.width, sd.camera.height)
        r = pi.render_guided(sc, g, spp=512, first_sample=100000)
        assert r.guide.guided_passes == 512 - 4 and r.guide.fallback == 0
        assert r.stats.nan_samples == 0
        g1, g2, gn = G.PathIntegrator.moments(gpu_ctx, sd.camera.width, sd.camera.height)
        assert (gn == 512).all()
        z = _block_z(g1, g2, gn, p1, p2, pn)
        zt = (g1.sum() / gn.sum() - p1.sum() / pn.sum())
        print(f"block |z| max {np.abs(z).max():.2f}, frac>3 {np.mean(np.abs(z) > 3):.3f}; image mean diff {zt:.4g}")
        assert np.mean(np.abs(z) > 3) < 0.03
        assert np.abs(z).max() < 6
    finally:
        g.close()
        sc.close()


@pytest.mark.parametrize("placement", ["continuation only", "next-event only"])
def test_guided_placements_are_unbiased(gpu_ctx, placement):
    """Either head alone (the other strategy a BSDF sample) keeps the estimate unbiased."""
    sd = _small_slit(64, 48)
    sc = G.Scene(gpu_ctx, sd)
    npix = sd.camera.width * sd.camera.height
    flags = A.BG_GUIDE_NO_NEE if placement == "continuation only" else A.BG_GUIDE_NO_CONTINUATION
    g = G.Guide(gpu_ctx, batch_size=4096, samples_per_pass=16384, warmup_passes=4, no_fallback=True, pass_paths=npix,
                flags=flags)
    try:
        pi = G.PathIntegrator(sd.camera, 512, sd.max_depth, mode=A.BG_MODE_PBRT, seed=8)
        pi.render(sc, spp=512)
        p1, p2, pn = G.PathIntegrator.moments(gpu_ctx, sd.camera.width, sd.camera.height)
        r = pi.render_guided(sc, g, spp=512, first_sample=200000)
        assert r.guide.guided_passes == 512 - 4 and r.stats.nan_samples == 0 and r.stats.error_word == 0
        g1, g2, gn = G.PathIntegrator.moments(gpu_ctx, sd.camera.width, sd.camera.height)
        z = _block_z(g1, g2, gn, p1, p2, pn)
        print(placement, f"block |z| max {np.abs(z).max():.2f}, frac>3 {np.mean(np.abs(z) > 3):.3f}")
        assert np.mean(np.abs(z) > 3) < 0.03
        assert np.abs(z).max() < 6
    finally:
        g.close()
        sc.close()


def _relmse(img, ref):
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))


def test_trained_guide_beats_bsdf_sampling(gpu_ctx):
    """Equal spp on the slit room: the guided estimate has lower relMSE than plain BSDF sampling."""
    sd = _small_slit(96, 64, depth=8)
    sc = G.Scene(gpu_ctx, sd)
    npix = sd.camera.width * sd.camera.height
    g = G.Guide(gpu_ctx, batch_size=4096, samples_per_pass=16384, warmup_passes=8, no_fallback=True, pass_paths=4 * npix,
                epochs=2)
    try:
        pi = G.PathIntegrator(sd.camera, 256, sd.max_depth, mode=A.BG_MODE_PBRT, seed=9)
        ref = pi.render(sc, spp=16384, first_sample=1 << 20).rgb
        plain = pi.render(sc, spp=256).rgb
        # train first, then measure a fresh guided render with the trained network
        pi.render_guided(sc, g, spp=256, first_sample=1 << 18)
        guided = pi.render_guided(sc, g, spp=256, first_sample=1 << 19)
        e_p, e_g = _relmse(plain, ref), _relmse(guided.rgb, ref)
        print(f"relMSE at 256 spp: plain {e_p:.4g}, guided {e_g:.4g} (ratio {e_g / e_p:.3f}); "
              f"relvar/sample plain {guided.guide.relvar_plain:.3g} guided {guided.guide.relvar_guided:.3g}")
        assert e_g < e_p
    finally:
        g.close()
        sc.close()


def test_multi_spp_passes_and_pool_export(gpu_ctx):
    """Passes of several spp: every pixel gets exactly spp samples, the exported pool holds sane
    training samples (unit directions, positions in [0,1], positive weights)."""
    sd = _small_slit(64, 48)
    sc = G.Scene(gpu_ctx, sd)
    npix = sd.camera.width * sd.camera.height
    g = G.Guide(gpu_ctx, batch_size=1024, samples_per_pass=8192, warmup_passes=2, no_fallback=True,
                pass_paths=3 * npix, epochs=3)
    try:
        pi = G.PathIntegrator(sd.camera, 20, sd.max_depth, mode=A.BG_MODE_PBRT, seed=2)
        r = pi.render_guided(sc, g, spp=20)
        assert r.guide.passes == 7 and r.guide.guided_passes == 5  # 3+3+...+2 spp
        _, _, n = G.PathIntegrator.moments(gpu_ctx, sd.camera.width, sd.camera.height)
        assert (n == 20).all()
        pool = g.pool()
        assert 0 < len(pool) <= 8192
        assert ((pool[:, :3] >= 0) & (pool[:, :3] <= 1)).all()
        for a, b in ((3, 6), (6, 9), (9, 12)):
            np.testing.assert_allclose(np.linalg.norm(pool[:, a:b], axis=1), 1.0, atol=1e-4)
        w = pool[:, 13:15]
        assert np.isfinite(w).all() and (w >= 0).all() and (w.max(axis=1) > 0).all() and (pool[:, 12] >= 0).all()
        assert (w[:, 0] > 0).any() and (w[:, 1] > 0).any()  # both heads get training samples
        assert r.guide.adam_steps == 7 * 3 * 8 or r.guide.adam_steps > 0
    finally:
        g.close()
        sc.close()


@pytest.mark.parametrize("scene", ["example", "textured"])
def test_guided_render_with_textures_infinite_light_and_strata_is_unbiased(gpu_ctx, scene):
    """Guided renders of the reference's example scene (UV texture, infinite light and two area
    lights, 16 x 16 stratified sampler) and of the textured room (image textures filtered with
    ray differentials) agree with plain renders of the same scenes block by block."""
    if scene == "example":
        sd = S.env_sphere(64, 48, spp=256, max_depth=5, extra=True)
        smp = S.StratifiedSampler(16, 16, 4, True)
    else:
        sd = S.textured_room(64, 48, spp=256, max_depth=5)
        smp = None
    sc = G.Scene(gpu_ctx, sd)
    npix = sd.camera.width * sd.camera.height
    g = G.Guide(gpu_ctx, batch_size=4096, samples_per_pass=16384, warmup_passes=4, no_fallback=True, pass_paths=npix)
    try:
        pi = G.PathIntegrator(sd.camera, 256, sd.max_depth, mode=A.BG_MODE_PBRT, seed=7, sampler=smp)
        pi.render(sc, spp=256)
        p1, p2, pn = G.PathIntegrator.moments(gpu_ctx, sd.camera.width, sd.camera.height)
        r = pi.render_guided(sc, g, spp=256, first_sample=1 << 16)
        assert r.guide.guided_passes == 256 - 4
        assert r.stats.nan_samples == 0 and r.stats.error_word == 0
        g1, g2, gn = G.PathIntegrator.moments(gpu_ctx, sd.camera.width, sd.camera.height)
        z = _block_z(g1, g2, gn, p1, p2, pn)
        print(scene, f"block |z| max {np.abs(z).max():.2f}, frac>3 {np.mean(np.abs(z) > 3):.3f}")
        assert np.mean(np.abs(z) > 3) < 0.03
        assert np.abs(z).max() < 6
    finally:
        g.close()
        sc.close()

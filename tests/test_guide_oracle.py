"""CPU checks of the FP64 guiding-network oracle (oracle/guide.py): the analytic gradient against
central finite differences, the mixture density's normalisation, and the sampling routine against
the density it claims."""
import numpy as np
import pytest

from oracle import guide as O


def _raw(n, seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    raw = rng.normal(0.0, scale, (n, O.HEAD_OUT))
    raw[:, 3:40:5] = rng.uniform(-1.5, 4.0, (n, O.LOBES))  # log kappa inside the clamp range
    return raw


def _dirs(n, seed):
    v = np.random.default_rng(seed).normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def test_loss_grad_matches_finite_differences():
    n = 16
    raw = _raw(n, 1)
    wi = _dirs(n, 2)
    p_b = np.where(np.arange(n) % 4 == 0, 0.0, 0.2 + np.arange(n) * 0.05)
    wn = np.full(n, 1.0 / n)
    _, g = O.loss_grad(raw, wi, p_b, wn)
    eps = 1e-6
    for j in range(O.HEAD_OUT):
        rp, rm = raw.copy(), raw.copy()
        rp[:, j] += eps
        rm[:, j] -= eps
        fd = (O.loss_grad(rp, wi, p_b, wn)[0] - O.loss_grad(rm, wi, p_b, wn)[0]) / (2 * eps)
        np.testing.assert_allclose(g[:, j], fd, rtol=1e-5, atol=1e-8, err_msg=f"output {j}")


def test_batch_gradient_matches_finite_differences():
    p = O.init_params(3).astype(np.float64)
    s = O.random_samples(64, 4).astype(np.float64)
    g, _ = O.batch_loss_grad(p, s)
    rng = np.random.default_rng(5)
    # every layer's weights, its bias column and the output rows
    idx = []
    for l in range(O.LAYERS):
        fan = O.IN_USED if l == 0 else O.HID
        base = O.param_off(l)
        for _ in range(6):
            r = rng.integers(0, O.used_rows(l))
            c = rng.integers(0, fan)
            idx.append(base + r * O.K + c)
        idx.append(base + int(rng.integers(0, O.used_rows(l))) * O.K + fan)  # bias
    eps = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (O.batch_loss(pp, s) - O.batch_loss(pm, s)) / (2 * eps)
        assert abs(g[i] - fd) <= 1e-5 * max(1.0, abs(fd)), (i, g[i], fd)


def test_padding_gradients_are_zero():
    p = O.init_params(0).astype(np.float64)
    g, _ = O.batch_loss_grad(p, O.random_samples(256, 1))
    for l in range(O.LAYERS):
        W = g[O.param_off(l):O.param_off(l) + O.rows(l) * O.K].reshape(O.rows(l), O.K)
        fan = O.IN_USED if l == 0 else O.HID
        assert not W[O.used_rows(l):].any()
        assert not W[:, fan + 1:].any()


def test_mixture_density_integrates_to_one():
    raw = _raw(4, 7)
    # Fibonacci sphere quadrature
    m = 200000
    i = np.arange(m) + 0.5
    z = 1 - 2 * i / m
    phi = np.pi * (1 + 5 ** 0.5) * i
    r = np.sqrt(1 - z * z)
    w = np.stack([r * np.cos(phi), r * np.sin(phi), z], 1)
    for k in range(len(raw)):
        p = O.pdf(np.repeat(raw[k:k + 1], m, 0), w)
        assert abs(p.mean() * 4 * np.pi - 1.0) < 2e-3


def test_sampling_matches_density():
    raw = _raw(1, 11)
    n = 400000
    u = np.random.default_rng(12).random((n, 3))
    d = O.sample(np.repeat(raw, n, 0), u)
    np.testing.assert_allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-12)
    # compare the histogram over z-bands with the integrated density
    zb = np.linspace(-1, 1, 21)
    hist = np.histogram(d[:, 2], zb)[0] / n
    m = 400000
    i = np.arange(m) + 0.5
    z = 1 - 2 * i / m
    phi = np.pi * (1 + 5 ** 0.5) * i
    r = np.sqrt(1 - z * z)
    w = np.stack([r * np.cos(phi), r * np.sin(phi), z], 1)
    p = O.pdf(np.repeat(raw, m, 0), w) * 4 * np.pi / m
    expect = np.histogram(z, zb, weights=p)[0]
    assert np.abs(hist - expect).max() < 4e-3


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159265, 0.0])
    b = O.bf16(x)
    assert b[0] == 1.0 and b[1] == 1.0  # tie -> even
    assert b[2] == 1.0078125
    assert abs(b[3] + 3.140625) < 1e-12


def test_octave_reduction_is_exact():
    """The device encoding reduces each octave's angle in FP32 before its hardware sine and cosine:
    t = p 2^k and r = t - 2 rint(t / 2).  Both steps are exact for p in [0, 1], so sin(pi r) and
    cos(pi r) equal the oracle's sin(pi 2^k p) and cos(pi 2^k p) up to FP64 rounding."""
    rng = np.random.default_rng(3)
    p = np.concatenate([rng.random(20000), [0.0, 1.0, 0.5, 0.25, 1.0 - 2.0 ** -24, 2.0 ** -24, 0.3333333]])
    p = p.astype(np.float32)
    q = np.zeros((len(p), 9))
    q[:, 0] = p
    ref = O.encode(q)
    for k in range(O.OCTAVES):
        t = p * np.float32(1 << k)
        r = t - np.float32(2.0) * np.rint(np.float32(0.5) * t)
        assert r.dtype == np.float32 and np.abs(r).max() <= 1.0
        # r is exact: t - r is an even integer, recovered without rounding
        assert np.array_equal((t.astype(np.float64) - r.astype(np.float64)) % 2.0, np.zeros(len(p)))
        np.testing.assert_allclose(np.sin(np.pi * r.astype(np.float64)), ref[:, 2 * k], atol=1e-9)
        np.testing.assert_allclose(np.cos(np.pi * r.astype(np.float64)), ref[:, 2 * k + 1], atol=1e-9)

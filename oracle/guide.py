"""FP64 host evaluation of the guiding network - TEST INFRASTRUCTURE ONLY.

The test oracle for the tensor-core kernels of bonsai_gb300 (k_guide_infer, k_guide_train,
k_guide_adam) and for the mixture device functions (guide_parse / guide_pdf / guide_sample /
guide_loss_grad).  The reference has no learned component, so there is nothing of it to follow
here: this module restates the network, the von Mises-Fisher mixture and the loss as defined in
include/bonsai_gpu.h, in float64 NumPy.

``bf16=True`` rounds what the GPU rounds to BF16 (encoded inputs, weights, hidden activations and
backpropagated errors) so the remaining difference is FP32 accumulation order; ``bf16=False`` is
the exact FP64 evaluation against which the BF16 error is stated.
"""
from __future__ import annotations

import numpy as np

LAYERS = 5
K = 80
HID = 64
HEADS = 2
HEAD_OUT = 41   # per head: 8 lobes x (direction 3, log kappa, weight logit) + selection logit
OUT = HEADS * HEAD_OUT
OUT_ROWS = 96
LOBES = 8
OCTAVES = 12
IN_USED = 78
PARAMS = 4 * HID * K + OUT_ROWS * K
C_MAX = 0.95
LOGK_MIN, LOGK_MAX = -2.0, 8.0


def rows(l: int) -> int:
    return OUT_ROWS if l == LAYERS - 1 else HID


def used_rows(l: int) -> int:
    return OUT if l == LAYERS - 1 else HID


def param_off(l: int) -> int:
    return l * HID * K


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(x, np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def weights(params: np.ndarray) -> list[np.ndarray]:
    p = np.asarray(params, np.float64)
    return [p[param_off(l):param_off(l) + rows(l) * K].reshape(rows(l), K) for l in range(LAYERS)]


def encode(q: np.ndarray) -> np.ndarray:
    """q (n, 9): p.xyz in [0,1], n.xyz, wo.xyz -> x (n, 80) with the constant-1 bias column 78."""
    q = np.asarray(q, np.float64)
    n = len(q)
    x = np.zeros((n, K))
    for c in range(3):
        for k in range(OCTAVES):
            a = np.pi * q[:, c] * (1 << k)
            x[:, c * 2 * OCTAVES + 2 * k] = np.sin(a)
            x[:, c * 2 * OCTAVES + 2 * k + 1] = np.cos(a)
    x[:, 72:78] = q[:, 3:9]
    x[:, 78] = 1.0
    return x


def forward(params: np.ndarray, q: np.ndarray, bf16_sim: bool = False):
    """Returns (raw (n, 48), activations list [x0, h1..h4]) - each activation (n, 80)."""
    W = weights(params)
    rnd = bf16 if bf16_sim else (lambda a: np.asarray(a, np.float64))
    a = rnd(encode(q))
    acts = [a]
    for l in range(LAYERS):
        z = a @ rnd(W[l]).T
        if l == LAYERS - 1:
            return z, acts
        h = np.maximum(z, 0.0)
        a = np.zeros((len(q), K))
        a[:, :HID] = h
        a[:, HID] = 1.0
        a = rnd(a)
        acts.append(a)
    raise AssertionError


def parse(raw: np.ndarray):
    """One head's mixture from its raw outputs (n, >= 41)."""
    raw = np.asarray(raw, np.float64)
    lob = raw[:, :40].reshape(-1, LOBES, 5)
    d = lob[:, :, :3]
    ln = np.linalg.norm(d, axis=2, keepdims=True)
    mu = np.where(ln > 1e-20, d / np.maximum(ln, 1e-300), np.array([0.0, 0.0, 1.0]))
    lk0 = lob[:, :, 3]
    lk = np.clip(lk0, LOGK_MIN, LOGK_MAX)
    kap = np.exp(lk)
    logc = lk - np.log(2 * np.pi) - np.log(-np.expm1(-2.0 * kap))
    a = lob[:, :, 4]
    a = a - a.max(axis=1, keepdims=True)
    pi = np.exp(a)
    pi /= pi.sum(axis=1, keepdims=True)
    sig = 1.0 / (1.0 + np.exp(-raw[:, 40]))
    return dict(d=d, dlen=np.maximum(ln[:, :, 0], 1e-20), mu=mu, lk0=lk0, kap=kap, logc=logc, pi=pi,
                sig=sig, c=C_MAX * sig)


def log_q(m: dict, w: np.ndarray):
    """log of the mixture density at directions w (n, 3); also the per-lobe terms."""
    mw = np.einsum("nlk,nk->nl", m["mu"], w)
    lv = m["logc"] + m["kap"] * (mw - 1.0)
    t = np.log(m["pi"]) + lv
    mx = t.max(axis=1, keepdims=True)
    lq = mx[:, 0] + np.log(np.exp(t - mx).sum(axis=1))
    return lq, t, mw


def pdf(raw: np.ndarray, w: np.ndarray) -> np.ndarray:
    m = parse(raw)
    return np.exp(log_q(m, np.asarray(w, np.float64))[0])


def sample(raw: np.ndarray, u: np.ndarray) -> np.ndarray:
    """The device sampling routine in FP64: lobe from u0, cos theta from u1 (Jakob 2012), phi = 2 pi u2."""
    m = parse(raw)
    u = np.asarray(u, np.float64)
    n = len(u)
    cdf = np.cumsum(m["pi"], axis=1)
    k = np.full(n, LOBES - 1)
    for i in range(LOBES - 2, -1, -1):
        k = np.where(u[:, 0] < cdf[:, i], i, k)
    kap = m["kap"][np.arange(n), k]
    mu = m["mu"][np.arange(n), k]
    ct = 1.0 + np.log(u[:, 1] + (1.0 - u[:, 1]) * np.exp(-2.0 * kap)) / kap
    ct = np.clip(ct, -1.0, 1.0)
    st = np.sqrt(np.maximum(0.0, 1.0 - ct * ct))
    ph = 2.0 * np.pi * u[:, 2]
    sign = np.where(mu[:, 2] >= 0, 1.0, -1.0)
    a = -1.0 / (sign + mu[:, 2])
    b = mu[:, 0] * mu[:, 1] * a
    t = np.stack([1.0 + sign * mu[:, 0] ** 2 * a, sign * b, -sign * mu[:, 0]], 1)
    bt = np.stack([b, sign + mu[:, 1] ** 2 * a, -mu[:, 1]], 1)
    v = ct[:, None] * mu + st[:, None] * (np.cos(ph)[:, None] * t + np.sin(ph)[:, None] * bt)
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def loss_grad(raw: np.ndarray, wi: np.ndarray, p_b: np.ndarray, wn: np.ndarray, alpha: float = 0.5):
    """Per-sample loss -wn [alpha log(c q + (1-c) p_b) + (1-alpha) log q] of one head and
    d loss / d raw (n, 41)."""
    raw = np.asarray(raw, np.float64)[:, :HEAD_OUT]
    wi = np.asarray(wi, np.float64)
    p_b = np.asarray(p_b, np.float64)
    wn = np.asarray(wn, np.float64)
    n = len(raw)
    m = parse(raw)
    lq, t, mw = log_q(m, wi)
    c = m["c"]
    la = np.log(c) + lq
    with np.errstate(divide="ignore"):
        lb = np.where(p_b > 0, np.log((1.0 - c) * np.where(p_b > 0, p_b, 1.0)), -np.inf)
    lmix = np.logaddexp(la, lb)
    s = np.exp(la - lmix)
    dmdc = np.where(p_b > 0, np.exp(lq - lmix) - p_b * np.exp(-lmix), 1.0 / c)
    active = wn > 0
    loss = np.where(active, -wn * (alpha * lmix + (1 - alpha) * lq), 0.0)
    dlq = -wn * (alpha * s + (1 - alpha))
    dc = -wn * alpha * dmdc
    r = np.exp(t - lq[:, None])
    g = np.zeros((n, HEAD_OUT))
    kap, mu, dlen = m["kap"], m["mu"], m["dlen"]
    sc = dlq[:, None] * r * kap / dlen
    gd = sc[:, :, None] * (wi[:, None, :] - mw[:, :, None] * mu)
    kfree = (m["lk0"] > LOGK_MIN) & (m["lk0"] < LOGK_MAX)
    with np.errstate(over="ignore"):
        dn = 1.0 - 2.0 * kap / np.expm1(2.0 * kap)
    gk = np.where(kfree, dlq[:, None] * r * (dn + kap * (mw - 1.0)), 0.0)
    ga = dlq[:, None] * (r - m["pi"])
    lob = np.concatenate([gd, gk[:, :, None], ga[:, :, None]], axis=2).reshape(n, 40)
    g[:, :40] = lob
    g[:, 40] = dc * C_MAX * m["sig"] * (1.0 - m["sig"])
    g[~active] = 0.0
    return loss, g


def split_samples(samples: np.ndarray):
    """query, wi, BSDF pdf, and the target weights of the two heads (indirect, direct)."""
    s = np.asarray(samples, np.float64).reshape(-1, 16)
    return s[:, :9], s[:, 9:12], s[:, 12], s[:, 13:15]


def _norm_weights(w: np.ndarray) -> np.ndarray:
    """Each head's weights over the batch, normalised by their sum (non-positive ones dropped)."""
    w = np.where(np.isfinite(w) & (w > 0), w, 0.0)
    s = w.sum(axis=0)
    return np.where(s > 0, w / np.where(s > 0, s, 1.0), 0.0)


def heads_loss_grad(raw: np.ndarray, wi: np.ndarray, p_b: np.ndarray, wn: np.ndarray, alpha: float = 0.5):
    """Both heads' per-sample losses (summed) and d loss / d raw (n, OUT_ROWS)."""
    g = np.zeros((len(raw), OUT_ROWS))
    loss = np.zeros(len(raw))
    for h in range(HEADS):
        lh, gh = loss_grad(raw[:, HEAD_OUT * h:HEAD_OUT * (h + 1)], wi, p_b, wn[:, h], alpha)
        loss += lh
        g[:, HEAD_OUT * h:HEAD_OUT * (h + 1)] = gh
    return loss, g


def batch_loss_grad(params: np.ndarray, samples: np.ndarray, alpha: float = 0.5, bf16_sim: bool = False):
    """Gradient of the batch loss (each head's weights normalised by their sum) w.r.t. the padded
    parameters."""
    q, wi, p_b, w = split_samples(samples)
    wn = _norm_weights(w)
    raw, acts = forward(params, q, bf16_sim)
    loss, dz = heads_loss_grad(raw, wi, p_b, wn, alpha)
    rnd = bf16 if bf16_sim else (lambda a: a)
    W = weights(params)
    grad = np.zeros(PARAMS)
    dz = rnd(dz)
    for l in range(LAYERS - 1, -1, -1):
        gW = dz.T @ acts[l]  # (rows, 80)
        gW[used_rows(l):] = 0.0
        grad[param_off(l):param_off(l) + rows(l) * K] = gW.reshape(-1)
        if l == 0:
            break
        dh = dz @ rnd(W[l])  # (n, 80)
        mask = acts[l][:, :HID] > 0
        dz = np.zeros((len(q), HID))
        dz[:, :] = np.where(mask, dh[:, :HID], 0.0)
        dz = rnd(dz)
    return grad, float(loss.sum())


def batch_loss(params: np.ndarray, samples: np.ndarray, alpha: float = 0.5) -> float:
    q, wi, p_b, w = split_samples(samples)
    raw, _ = forward(params, q)
    loss, _ = heads_loss_grad(raw, wi, p_b, _norm_weights(w), alpha)
    return float(loss.sum())


def adam(params, m, v, g, t: int, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return params - lr * mh / (np.sqrt(vh) + eps), m, v


def init_params(seed: int = 0) -> np.ndarray:
    """A seeded parameter vector in the library's layout (He-uniform, zero biases and padding)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(PARAMS, np.float32)
    for l in range(LAYERS):
        fan = IN_USED if l == 0 else HID
        bound = np.sqrt(6.0 / fan) * (0.1 if l == LAYERS - 1 else 1.0)
        W = p[param_off(l):param_off(l) + rows(l) * K].reshape(rows(l), K)
        W[:used_rows(l), :fan] = rng.uniform(-bound, bound, (used_rows(l), fan))
        W[:used_rows(l), fan] = rng.uniform(-0.1, 0.1, used_rows(l))  # non-zero biases exercise the bias column
    return p


def random_samples(n: int, seed: int = 0) -> np.ndarray:
    """Seeded training samples: queries, unit wi, BSDF pdf (some zero) and heavy-tailed weights of
    both heads (some zero)."""
    rng = np.random.default_rng(seed)
    s = np.zeros((n, 16), np.float32)
    s[:, 0:3] = rng.random((n, 3))
    nrm = rng.normal(size=(n, 3))
    s[:, 3:6] = nrm / np.linalg.norm(nrm, axis=1, keepdims=True)
    wo = rng.normal(size=(n, 3))
    s[:, 6:9] = wo / np.linalg.norm(wo, axis=1, keepdims=True)
    wi = rng.normal(size=(n, 3))
    s[:, 9:12] = wi / np.linalg.norm(wi, axis=1, keepdims=True)
    s[:, 12] = np.where(rng.random(n) < 0.1, 0.0, rng.exponential(0.3, n))
    s[:, 13] = np.where(rng.random(n) < 0.2, 0.0, rng.lognormal(0.0, 1.0, n))
    s[:, 14] = np.where(rng.random(n) < 0.6, 0.0, rng.lognormal(0.5, 1.5, n))
    return s

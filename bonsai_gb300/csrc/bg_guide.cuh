// bg_guide.cuh - neural path guiding: network layout, input encoding, the von Mises-Fisher
// mixture it outputs, and the per-sample loss gradient.  No counterpart in the reference (its
// PathIntegrator samples the BSDF only); the estimator stays unbiased because every guided
// direction is weighted by the pdf of the one-sample mixture it was drawn from.
//
// Network: 78 inputs -> 4 hidden layers of 64 (ReLU) -> 2 heads of 41 outputs.
//   inputs  x[0..71]  position: each scene-normalised coordinate p in [0,1] through 12 octaves,
//                     x[24c + 2k] = sin(pi 2^k p_c), x[24c + 2k + 1] = cos(pi 2^k p_c)
//           x[72..74] shading normal, x[75..77] outgoing direction wo
//   outputs per head (head h at raw[41 h ..]): raw[5i .. 5i+2] lobe i mean direction
//           (normalised), raw[5i+3] log kappa, raw[5i+4] lobe weight logit (8 lobes), raw[40]
//           logit of the guide selection probability.  Head 0 proposes continuations (trained on
//           the indirect radiance along a direction), head 1 next-event directions (trained on
//           the emission a direction reaches).
// The parameter layout (biases folded into a constant-1 input column) is in bg_guide_layout.h.
#pragma once
#include <cuda_bf16.h>

#include "bg_guide_layout.h"
#include "bg_math.cuh"

namespace bg {

// Encoded input of one query (80 values, see above).  q: p.xyz (in [0,1]), n.xyz, wo.xyz.
// Each octave's angle is reduced exactly before the hardware sine / cosine: t = 2^k p is exact, and
// so is r = t - 2 rint(t / 2) in [-1, 1], with sin(pi t) = sin(pi r); __sinf / __cosf on [-pi, pi]
// are within 2^-21 of the true values, far below the BF16 rounding the network input gets.
BG_D void guide_encode(const float* q, float* x) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
#pragma unroll
        for (int k = 0; k < GUIDE_OCTAVES; ++k) {
            const float t = q[c] * (float)(1 << k);
            const float a = PI * (t - 2.0f * rintf(0.5f * t));
            x[c * 2 * GUIDE_OCTAVES + 2 * k] = __sinf(a);
            x[c * 2 * GUIDE_OCTAVES + 2 * k + 1] = __cosf(a);
        }
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) x[72 + i] = q[3 + i];
    x[78] = 1.0f;
    x[79] = 0.0f;
}

// ---------------------------------------------------------------- vMF mixture
constexpr float GUIDE_C_MAX = 0.95f;   // the BSDF keeps >= 5% of the proposal
constexpr float GUIDE_LOGK_MIN = -2.0f, GUIDE_LOGK_MAX = 8.0f;
constexpr float LOG_2PI = 1.8378770664093453f;

// log(1 - e^{-2 kappa}) without cancellation for small kappa
BG_D float vmf_log_norm(float kappa, float logk) { return logk - LOG_2PI - __logf(-expm1f(-2.0f * kappa)); }

// Direction from one vMF lobe: cos(theta) = 1 + log(u1 + (1 - u1) e^{-2 kappa}) / kappa
// (W. Jakob, "Numerically stable sampling of the von Mises-Fisher distribution on S^2", 2012) and
// phi = 2 pi u2.
BG_D V3 vmf_sample_lobe(V3 mu, float kappa, float u1, float u2) {
    float ct = 1.0f + __logf(u1 + (1.0f - u1) * __expf(-2.0f * kappa)) / kappa;
    ct = rclamp(ct, -1.0f, 1.0f);
    float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
    float sp, cp;
    sincospif(2.0f * u2, &sp, &cp);
    // orthonormal basis around mu (T. Duff et al., "Building an orthonormal basis, revisited", JCGT 2017)
    float sign = copysignf(1.0f, mu.z);
    float a = -1.0f / (sign + mu.z);
    float b = mu.x * mu.y * a;
    V3 t = v3(1.0f + sign * mu.x * mu.x * a, sign * b, -sign * mu.x);
    V3 bt = v3(b, sign + mu.y * mu.y * a, -mu.y);
    return normalize(ct * mu + st * (cp * t + sp * bt));
}

// Concentration and mean direction of a stored lobe b = kappa mu, with every operation rounded as
// written: the inference epilogue and the shade kernels (compiled with and without contraction)
// derive bit-identical values, so the density the sampler draws from is the one the pdf evaluates.
BG_D float mix_kappa(float4 l) {
    return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(l.x, l.x), __fmul_rn(l.y, l.y)), __fmul_rn(l.z, l.z)));
}

// Mixture record of one head (41 raw outputs) as stored by the render-side inference
// (GUIDE_MIX_HEAD floats): per lobe b = kappa mu and a = log w + log c(kappa) - kappa, with kappa
// re-derived from the stored b (mix_kappa), then the running lobe-weight sums and c.
//   mu = d / |d| of the lobe's three direction outputs d (d ~ 0: +z), kappa = exp(clamped log
//   kappa), w = softmax of the eight weight logits, c(kappa) = kappa / (2 pi (1 - e^{-2 kappa})),
//   c = 0.95 sigmoid(selection logit).
// log w comes from the logits directly (logit - max - log sum); 1 - e^{-2 kappa} needs no expm1
// here because kappa >= e^-2 keeps it above 0.23.
BG_D void guide_write_mixture(const float* raw, float* out) {
    float mx = -FLT_BIG;
#pragma unroll
    for (int i = 0; i < GUIDE_LOBES; ++i) mx = fmaxf(mx, raw[5 * i + 4]);
    float e[GUIDE_LOBES], sum = 0.0f;
#pragma unroll
    for (int i = 0; i < GUIDE_LOBES; ++i) {
        e[i] = __expf(raw[5 * i + 4] - mx);
        sum += e[i];
    }
    const float inv = 1.0f / sum, lsum = __logf(sum);
    float acc = 0.0f;
#pragma unroll
    for (int i = 0; i < GUIDE_LOBES; ++i) {
        const float dx = raw[5 * i], dy = raw[5 * i + 1], dz = raw[5 * i + 2];
        const float l2 = dx * dx + dy * dy + dz * dz;
        const float kap = __expf(rclamp(raw[5 * i + 3], GUIDE_LOGK_MIN, GUIDE_LOGK_MAX));
        float4 l = make_float4(0.0f, 0.0f, kap, 0.0f);
        if (l2 > 1e-30f) {
            const float sc = kap * rsqrtf(l2);
            l = make_float4(sc * dx, sc * dy, sc * dz, 0.0f);
        }
        const float k = mix_kappa(l);
        l.w = (raw[5 * i + 4] - mx - lsum) + __logf(k) - LOG_2PI - __logf(1.0f - __expf(-2.0f * k)) - k;
        out[4 * i] = l.x;
        out[4 * i + 1] = l.y;
        out[4 * i + 2] = l.z;
        out[4 * i + 3] = l.w;
        acc += e[i] * inv;
        if (i < GUIDE_LOBES - 1) out[32 + i] = acc;
    }
    out[39] = GUIDE_C_MAX / (1.0f + __expf(-raw[40]));
}

// Read-only view of one head's stored mixture: lobes are loaded as they are needed, so a kernel
// does not keep the whole mixture in registers.  pdf(w) = sum_i exp(a_i + b_i . w).
struct MixView {
    const float* m;
    BG_D float c() const { return m[39]; }
    BG_D float pdf(V3 w) const {
        float p = 0.0f;
#pragma unroll 4
        for (int i = 0; i < GUIDE_LOBES; ++i) {
            const float4 l = *reinterpret_cast<const float4*>(m + 4 * i);
            p += __expf(l.w + l.x * w.x + l.y * w.y + l.z * w.z);
        }
        return p;
    }
    BG_D V3 sample(float u0, float u1, float u2) const {
        int k = GUIDE_LOBES - 1;
        for (int i = 0; i < GUIDE_LOBES - 1; ++i)
            if (u0 < m[32 + i]) {
                k = i;
                break;
            }
        const float4 l = *reinterpret_cast<const float4*>(m + 4 * k);
        const float kap = mix_kappa(l);
        const V3 mu = v3(__fdiv_rn(l.x, kap), __fdiv_rn(l.y, kap), __fdiv_rn(l.z, kap));
        return vmf_sample_lobe(mu, kap, u1, u2);
    }
};

// ---------------------------------------------------------------- training loss
// Per sample (direction wi drawn from the proposal that rendered it, p_b = BSDF pdf of wi,
// weight w = f(wo, wi) |cos| Li(wi) / p_proposal(wi) as luminance, wn = w / sum of w over the batch):
//   loss = -wn [alpha log(c q(wi) + (1 - c) p_b) + (1 - alpha) log q(wi)]
// a Monte Carlo estimate of the KL divergence from the normalised product f Li cos to the
// one-sample mixture (first term) and to the guide alone (second term), up to a constant.
// `raw` is one head's 41 outputs; writes d loss / d raw (41 values) and returns the loss.
constexpr float GUIDE_ALPHA = 0.5f;

BG_D float guide_loss_grad(const float* raw, V3 wi, float p_b, float wn, float alpha, float* g) {
#pragma unroll
    for (int j = 0; j < GUIDE_HEAD_OUT; ++j) g[j] = 0.0f;
    if (!(wn > 0.0f)) return 0.0f;
    float mx = -FLT_BIG;
#pragma unroll
    for (int i = 0; i < GUIDE_LOBES; ++i) mx = fmaxf(mx, raw[5 * i + 4]);
    float pi_[GUIDE_LOBES], lv[GUIDE_LOBES], kap[GUIDE_LOBES], mw[GUIDE_LOBES], dlen[GUIDE_LOBES];
    V3 mu[GUIDE_LOBES];
    bool kfree[GUIDE_LOBES];
    float psum = 0.0f;
    float lmax = -FLT_BIG;
#pragma unroll
    for (int i = 0; i < GUIDE_LOBES; ++i) {
        V3 d = v3(raw[5 * i], raw[5 * i + 1], raw[5 * i + 2]);
        float l = length(d);
        dlen[i] = fmaxf(l, 1e-20f);
        mu[i] = l > 1e-20f ? d / l : v3(0.0f, 0.0f, 1.0f);
        float lk0 = raw[5 * i + 3];
        kfree[i] = lk0 > GUIDE_LOGK_MIN && lk0 < GUIDE_LOGK_MAX;
        float lk = rclamp(lk0, GUIDE_LOGK_MIN, GUIDE_LOGK_MAX);
        kap[i] = __expf(lk);
        mw[i] = dot(mu[i], wi);
        lv[i] = vmf_log_norm(kap[i], lk) + kap[i] * (mw[i] - 1.0f);
        pi_[i] = __expf(raw[5 * i + 4] - mx);
        psum += pi_[i];
    }
    float lq_terms[GUIDE_LOBES];
#pragma unroll
    for (int i = 0; i < GUIDE_LOBES; ++i) {
        pi_[i] = pi_[i] / psum;
        lq_terms[i] = __logf(pi_[i]) + lv[i];
        lmax = fmaxf(lmax, lq_terms[i]);
    }
    float se = 0.0f;
#pragma unroll
    for (int i = 0; i < GUIDE_LOBES; ++i) se += __expf(lq_terms[i] - lmax);
    const float lq = lmax + __logf(se);  // log q(wi)
    const float sig = 1.0f / (1.0f + __expf(-raw[40]));
    const float c = GUIDE_C_MAX * sig;
    // log mix, s = c q / mix, dmix_dc = (q - p_b) / mix, all in log space
    const float la = __logf(c) + lq;
    float lmix, s, dmdc;
    if (p_b > 0.0f) {
        float lb = __logf((1.0f - c) * p_b);
        float hi = fmaxf(la, lb);
        lmix = hi + log1pf(__expf(-fabsf(la - lb)));
        s = __expf(la - lmix);
        dmdc = __expf(lq - lmix) - __expf(__logf(p_b) - lmix);
    } else {
        lmix = la;
        s = 1.0f;
        dmdc = 1.0f / c;
    }
    const float loss = -wn * (alpha * lmix + (1.0f - alpha) * lq);
    const float dlq = -wn * (alpha * s + (1.0f - alpha));  // d loss / d log q
    const float dc = -wn * alpha * dmdc;                    // d loss / d c
#pragma unroll
    for (int i = 0; i < GUIDE_LOBES; ++i) {
        float r = __expf(lq_terms[i] - lq);  // responsibility pi_i v_i / q
        // direction: d log v / d d = kappa (wi - (mu.wi) mu) / |d|
        float sc = dlq * r * kap[i] / dlen[i];
        g[5 * i + 0] = sc * (wi.x - mw[i] * mu[i].x);
        g[5 * i + 1] = sc * (wi.y - mw[i] * mu[i].y);
        g[5 * i + 2] = sc * (wi.z - mw[i] * mu[i].z);
        // log kappa: d log v / d log kappa = 1 - 2 kappa / (e^{2 kappa} - 1) + kappa (mu.wi - 1)
        if (kfree[i]) {
            float dn = 1.0f - 2.0f * kap[i] / expm1f(2.0f * kap[i]);
            g[5 * i + 3] = dlq * r * (dn + kap[i] * (mw[i] - 1.0f));
        }
        // softmax logits: d log q / d a_i = r_i - pi_i
        g[5 * i + 4] = dlq * (r - pi_[i]);
    }
    g[40] = dc * GUIDE_C_MAX * sig * (1.0f - sig);
    return loss;
}

}  // namespace bg

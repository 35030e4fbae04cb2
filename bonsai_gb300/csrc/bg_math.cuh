// bg_math.cuh - device arithmetic for the path-tracing kernels (sm_103a).
//
// All translation units are compiled with -fmad=false: every + - * / is rounded as written, the
// f32 semantics of the reference (kazijawad/bonsai is Rust, which never contracts).  fmaf() is
// used explicitly only where an exact product error is wanted (error-free transformations) and
// in the slab tests of the wide BVH, which has no reference counterpart.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "bg_device.h"

#define BG_HD __host__ __device__ __forceinline__
#define BG_D __device__ __forceinline__

namespace bg {

constexpr float PI = 3.14159265358979323846f;
constexpr float PI_OVER_TWO = PI / 2.0f;
constexpr float INV_PI = 1.0f / PI;
constexpr float FLT_EPS = 1.1920928955078125e-07f;
constexpr float MACHINE_EPSILON = FLT_EPS * 0.5f;
constexpr float ONE_MINUS_EPSILON = 1.0f - FLT_EPS;
constexpr float FLT_BIG = 3.40282347e+38f;

// src/base/math.rs:3-5, evaluated in f32 like the reference
BG_HD float gamma(float n) { return (n * MACHINE_EPSILON) / (1.0f - n * MACHINE_EPSILON); }

BG_D float next_float_up(float v) {  // src/base/math.rs:27-41
    if (isinf(v) && v > 0.0f) return v;
    if (v == -0.0f) v = 0.0f;
    uint32_t ui = __float_as_uint(v);
    ui = (v >= 0.0f) ? ui + 1 : ui - 1;
    return __uint_as_float(ui);
}
BG_D float next_float_down(float v) {  // src/base/math.rs:11-25
    if (isinf(v) && v < 0.0f) return v;
    if (v == 0.0f) v = -0.0f;
    uint32_t ui = __float_as_uint(v);
    ui = (v > 0.0f) ? ui - 1 : ui + 1;
    return __uint_as_float(ui);
}
BG_D float rmin(float a, float b) { return fminf(a, b); }
BG_D float rmax(float a, float b) { return fmaxf(a, b); }
BG_D float rclamp(float v, float lo, float hi) {
    if (v < lo) v = lo;
    if (v > hi) v = hi;
    return v;
}

// a*b - c*d with the products' rounding errors recovered by fma (Kahan's difference of
// products, W. Kahan / Jeannerod et al. 2013).  Replaces the reference's f64 evaluation of
// edge functions (src/shapes/triangle.rs:179-190) and cross products (src/geometries/vec3.rs:108-122):
// the sign is exact and the value is within 1.5 ulp of the exact difference.
BG_D float diff_of_products(float a, float b, float c, float d) {
    float cd = __fmul_rn(c, d);
    float err = fmaf(-c, d, cd);
    float dop = fmaf(a, b, -cd);
    return __fadd_rn(dop, err);
}

struct V3 {
    float x, y, z;
};
BG_D V3 v3(float x, float y, float z) { return V3{x, y, z}; }
BG_D V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
BG_D V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
BG_D V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
BG_D V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
BG_D V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
BG_D V3 operator/(V3 a, float s) {  // multiply by the reciprocal, src/geometries/vec3.rs:330-342
    float inv = 1.0f / s;
    return {a.x * inv, a.y * inv, a.z * inv};
}
BG_D float get(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
BG_D void set(V3& a, int i, float v) {
    if (i == 0) a.x = v;
    else if (i == 1) a.y = v;
    else a.z = v;
}
BG_D float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
BG_D float abs_dot(V3 a, V3 b) { return fabsf(dot(a, b)); }
BG_D V3 vabs(V3 a) { return {fabsf(a.x), fabsf(a.y), fabsf(a.z)}; }
BG_D float length_squared(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
BG_D float length(V3 a) { return sqrtf(length_squared(a)); }
BG_D V3 normalize(V3 a) { return a / length(a); }
BG_D V3 cross(V3 a, V3 b) {
    return {diff_of_products(a.y, b.z, a.z, b.y), diff_of_products(a.z, b.x, a.x, b.z),
            diff_of_products(a.x, b.y, a.y, b.x)};
}
BG_D float max_component(V3 a) { return rmax(a.x, rmax(a.y, a.z)); }
BG_D int max_dimension(V3 a) {
    if (a.x > a.y) return a.x > a.z ? 0 : 2;
    return a.y > a.z ? 1 : 2;
}
BG_D V3 permute(V3 a, int x, int y, int z) { return {get(a, x), get(a, y), get(a, z)}; }
BG_D V3 face_forward(V3 n, V3 v) { return dot(n, v) < 0.0f ? -n : n; }
BG_D float distance_squared(V3 a, V3 b) { return length_squared(a - b); }
BG_D V3 f4xyz(float4 f) { return {f.x, f.y, f.z}; }

// RGBSpectrum (src/spectra/rgb.rs)
struct RGB {
    float r, g, b;
};
BG_D RGB rgb(float v) { return {v, v, v}; }
BG_D RGB rgb(float r, float g, float b) { return {r, g, b}; }
BG_D RGB operator+(RGB a, RGB b) { return {a.r + b.r, a.g + b.g, a.b + b.b}; }
BG_D RGB operator-(RGB a, RGB b) { return {a.r - b.r, a.g - b.g, a.b - b.b}; }
BG_D RGB operator*(RGB a, RGB b) { return {a.r * b.r, a.g * b.g, a.b * b.b}; }
BG_D RGB operator/(RGB a, RGB b) { return {a.r / b.r, a.g / b.g, a.b / b.b}; }
BG_D RGB operator*(RGB a, float s) { return {a.r * s, a.g * s, a.b * s}; }
BG_D RGB operator*(float s, RGB a) { return {s * a.r, s * a.g, s * a.b}; }
BG_D RGB operator/(RGB a, float s) {
    float inv = 1.0f / s;
    return {a.r * inv, a.g * inv, a.b * inv};
}
BG_D bool is_black(RGB a) { return a.r == 0.0f && a.g == 0.0f && a.b == 0.0f; }
BG_D bool is_nan(RGB a) { return isnan(a.r) || isnan(a.g) || isnan(a.b); }
BG_D float max_value(RGB a) { return rmax(rmax(a.r, a.g), a.b); }
BG_D float luminance(RGB a) { return 0.212671f * a.r + 0.715160f * a.g + 0.072169f * a.b; }
BG_D RGB rgb_sqrt(RGB a) { return {sqrtf(a.r), sqrtf(a.g), sqrtf(a.b)}; }

// EFloat (src/base/efloat.rs)
struct EF {
    float v, lo, hi;
};
BG_D EF ef(float v, float err) {
    if (err == 0.0f) return {v, v, v};
    return {v, next_float_down(v - err), next_float_up(v + err)};
}
BG_D EF ef(float v) { return {v, v, v}; }
BG_D EF operator+(EF a, EF b) { return {a.v + b.v, next_float_down(a.lo + b.lo), next_float_up(a.hi + b.hi)}; }
BG_D EF operator-(EF a, EF b) { return {a.v - b.v, next_float_down(a.lo - b.hi), next_float_up(a.hi - b.lo)}; }
BG_D EF operator*(EF a, EF b) {
    float p0 = a.lo * b.lo, p1 = a.hi * b.lo, p2 = a.lo * b.hi, p3 = a.hi * b.hi;
    return {a.v * b.v, next_float_down(rmin(rmin(rmin(p0, p1), p2), p3)),
            next_float_up(rmax(rmax(rmax(p0, p1), p2), p3))};
}
BG_D EF operator/(EF a, EF b) {
    float q0 = a.lo / b.lo, q1 = a.hi / b.lo, q2 = a.lo / b.hi, q3 = a.hi / b.hi;
    bool straddle = b.lo < 0.0f && b.hi > 0.0f;
    float lo = straddle ? -INFINITY : next_float_down(rmin(rmin(rmin(q0, q1), q2), q3));
    float hi = straddle ? INFINITY : next_float_up(rmax(rmax(rmax(q0, q1), q2), q3));
    return {a.v / b.v, lo, hi};
}
// EFloat::quadratic (src/base/efloat.rs:36-67).  The reference evaluates the discriminant in f64;
// here b*b - 4ac is formed from exact fma product splits (no f64 on the device):
// D = (bb_hi - ac4_hi) + (bb_lo - ac4_lo), with 4ac exact because scaling by 4 is exact.
BG_D bool quadratic(EF a, EF b, EF c, EF* t0, EF* t1) {
    float bb = b.v * b.v;
    float bb_lo = fmaf(b.v, b.v, -bb);
    float ac = a.v * c.v;
    float ac_lo = fmaf(a.v, c.v, -ac);
    float ac4 = 4.0f * ac, ac4_lo = 4.0f * ac_lo;
    float d_hi = bb - ac4;
    float d = d_hi + (bb_lo - ac4_lo);
    if (d < 0.0f) return false;
    float root = sqrtf(d);
    EF rootf = ef(root, MACHINE_EPSILON * root);
    EF q = (b.v < 0.0f) ? ef(-0.5f) * (b - rootf) : ef(-0.5f) * (b + rootf);
    *t0 = q / a;
    *t1 = c / q;
    if (t0->v > t1->v) {
        EF t = *t0;
        *t0 = *t1;
        *t1 = t;
    }
    return true;
}

// ---- counter-based RNG: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
// key = {pixel, seed.lo}, counter = {sample, dim/4, seed.hi, 0x626F6E73}; lane dim%4;
// uniform = (u >> 9) * 2^-23 (the value grid of rand 0.8's Uniform<f32>(0..1)).
BG_HD void philox4x32_10(uint32_t ctr[4], uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * ctr[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * ctr[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ ctr[1] ^ k0, n2 = hi0 ^ ctr[3] ^ k1;
        ctr[0] = n0;
        ctr[1] = lo1;
        ctr[2] = n2;
        ctr[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}
struct Rng {
    uint32_t pixel, sample;
    uint64_t seed;
    uint32_t stream;  // 0 for path integrators; a tree integrator's node (node id - 1)
    // four consecutive dimensions starting at a multiple of 4
    BG_D void block(uint32_t dim4, float out[4]) const {
        uint32_t c[4] = {sample, dim4 >> 2, (uint32_t)(seed >> 32), 0x626F6E73u ^ stream};
        philox4x32_10(c, pixel, (uint32_t)seed);
#pragma unroll
        for (int i = 0; i < 4; ++i) out[i] = (float)(c[i] >> 9) * 0x1p-23f;
    }
    BG_D float u(uint32_t dim) const {
        float b[4];
        block(dim & ~3u, b);
        return b[dim & 3];
    }
    BG_D uint32_t bits(uint32_t dim) const {  // the raw 32 bits behind u(dim)
        uint32_t c[4] = {sample, dim >> 2, (uint32_t)(seed >> 32), 0x626F6E73u ^ stream};
        philox4x32_10(c, pixel, (uint32_t)seed);
        return c[dim & 3];
    }
};

// The pixel of a render's linear pixel index t in [0, w * h): scanline order, or (tiles != 0)
// bands of 4 rows walked in 8 x 4 tiles, so that the 32 camera rays of a warp cover a compact block;
// the ragged right column of tiles (w % 8) and bottom band (h % 4) keep narrower / shorter tiles.
BG_HD uint32_t pixel_of(uint32_t t, uint32_t w, uint32_t h, uint32_t tiles) {
    if (!tiles) return t;
    const uint32_t full_band = 4u * w, nfull = h / 4u;
    const uint32_t band = t / full_band < nfull ? t / full_band : nfull;
    const uint32_t y0 = band * 4u, bh = band < nfull ? 4u : h - y0;
    const uint32_t o = t - band * full_band;
    const uint32_t wt = w / 8u, tile = 8u * bh;
    uint32_t x, y;
    if (o < wt * tile) {
        const uint32_t c = o / tile, k = o - c * tile;
        x = c * 8u + (k & 7u);
        y = y0 + (k >> 3);
    } else {
        const uint32_t r = o - wt * tile, wr = w - wt * 8u;
        x = wt * 8u + r % wr;
        y = y0 + r / wr;
    }
    return y * w + x;
}

// Dimension schedule shared with the CPU oracle: camera film.xy 0-1, lens 2-3, time 4;
// bounce b: base 8+8b: light pick +0, u_light +1..2, u_scattering +3..4, BSDF +5..6, roulette +7.
constexpr uint32_t DIM_FILM = 0, DIM_TIME = 4, DIM_BOUNCE0 = 8, DIMS_PER_BOUNCE = 8;
constexpr uint32_t BD_LIGHT = 0, BD_ULIGHT = 1, BD_USCAT = 3, BD_BSDF = 5, BD_RR = 7;

// ---- StratifiedSampler (src/samplers/stratified.rs:75-137, src/base/sampling.rs:120-179) without
// per-pixel arrays.  The samples of a pixel form passes of spp = nx * ny (pass = sample / spp); in
// each pass, stratified dimension k of sample s takes stratum perm_k(s % spp), jittered inside the
// stratum (1D: spp strata of [0, 1); 2D: an nx x ny grid).  perm_k is the identity in REF_COMPAT
// mode (F6: shuffle never swaps, so every dimension walks the strata in the same order) and a
// keyed permutation in PBRT mode.  Random numbers come from the counter RNG on stream
// 0x80000000 | 2k | is_2d: dimension 0 keys the permutation, 4 + 2j and 5 + 2j jitter stratum j.
// A bijection of [0, n) keyed by `key`: a keyed bijection of [0, 2^b) (xor, odd multiply, xorshift,
// add; each invertible modulo 2^b) iterated until it lands below n (cycle walking: the cycle through
// i < n returns to [0, n) within 2^b steps).
BG_HD uint32_t strat_permute(uint32_t i, uint32_t n, uint32_t key) {
    if (n <= 1) return 0;
    uint32_t b = 0;
    while ((1u << b) < n) ++b;
    const uint32_t mask = b >= 32 ? 0xFFFFFFFFu : (1u << b) - 1u;
    const uint32_t sh = (b + 1) / 2;
    uint32_t x = i;
    for (uint32_t it = 0; it <= mask; ++it) {
        x = (x ^ key) & mask;
        x = (x * 0x2F5A6B1Du) & mask;
        x ^= x >> sh;
        x = (x + (key >> 7)) & mask;
        x = (x * 0x6C8E9CF5u) & mask;
        x ^= x >> sh;
        x = (x ^ (key >> 13) ^ 0x5BD1E995u) & mask;
        x = (x * 0x1B873593u) & mask;
        x ^= x >> sh;
        if (x < n) return x;
    }
    return i;  // not reached
}
BG_D uint32_t strat_stratum(const StratParams& sp, bool ref, uint32_t pix, uint32_t sample, uint64_t seed, uint32_t k,
                            uint32_t is2d, Rng* jr) {
    const uint32_t n = sp.nx * sp.ny;
    const uint32_t s = sample % n;
    *jr = Rng{pix, sample / n, seed, 0x80000000u | (k << 1) | is2d};
    return ref ? s : strat_permute(s, n, jr->bits(0));
}
// get_1d / get_2d for stratified dimension k (k < sp.dims).
BG_D float strat_1d(const StratParams& sp, bool ref, uint32_t pix, uint32_t sample, uint64_t seed, uint32_t k) {
    Rng jr;
    const uint32_t j = strat_stratum(sp, ref, pix, sample, seed, k, 0u, &jr);
    const float delta = sp.jitter ? jr.u(4 + 2 * j) : 0.5f;
    const float inv = 1.0f / (float)(sp.nx * sp.ny);
    return rmin(((float)j + delta) * inv, ONE_MINUS_EPSILON);
}
BG_D float2 strat_2d(const StratParams& sp, bool ref, uint32_t pix, uint32_t sample, uint64_t seed, uint32_t k) {
    Rng jr;
    const uint32_t j = strat_stratum(sp, ref, pix, sample, seed, k, 1u, &jr);
    const float jx = sp.jitter ? jr.u(4 + 2 * j) : 0.5f, jy = sp.jitter ? jr.u(5 + 2 * j) : 0.5f;
    const float dx = 1.0f / (float)sp.nx, dy = 1.0f / (float)sp.ny;
    return make_float2(rmin(((float)(j % sp.nx) + jx) * dx, ONE_MINUS_EPSILON),
                       rmin(((float)(j / sp.nx) + jy) * dy, ONE_MINUS_EPSILON));
}
// A sample's sampler calls in the reference's order: get_1d / get_2d number k1 / k2 take stratified
// values while below sp.dims and otherwise keep the counter RNG's value already in place.
struct SamplerCalls {
    const StratParams& sp;
    bool ref;
    uint32_t pix, sample;
    uint64_t seed;
    uint32_t k1, k2;
    BG_D void get_1d(float& v) {
        if (k1 < sp.dims) v = strat_1d(sp, ref, pix, sample, seed, k1);
        ++k1;
    }
    BG_D void get_2d(float& a, float& b) {
        if (k2 < sp.dims) {
            const float2 t = strat_2d(sp, ref, pix, sample, seed, k2);
            a = t.x;
            b = t.y;
        }
        ++k2;
    }
};
// The sampler calls a camera sample makes (Sampler::get_camera_sample: film get_2d, lens get_2d,
// time get_1d): the film offset and the time, from the stratified sampler or the counter RNG.
struct CameraUs {
    float fx, fy, time;
    float lx, ly;  // lens sample
};
// lens / time: whether the caller needs the lens sample (a thin-lens camera) and the time.
BG_D CameraUs camera_us(const StratParams& sp, bool ref, const Rng& rng, bool lens, bool time = true) {
    CameraUs c;
    c.lx = c.ly = 0.5f;
    c.time = 0.0f;
    if (sp.dims == 0) {
        float b[4];
        rng.block(0, b);  // film 0-1, lens 2-3
        c.fx = b[0];
        c.fy = b[1];
        if (lens) {
            c.lx = b[2];
            c.ly = b[3];
        }
        if (time) c.time = rng.u(DIM_TIME);
        return c;
    }
    const float2 f = strat_2d(sp, ref, rng.pixel, rng.sample, rng.seed, 0);
    c.fx = f.x;
    c.fy = f.y;
    if (time) c.time = strat_1d(sp, ref, rng.pixel, rng.sample, rng.seed, 0);
    if (lens) {
        if (sp.dims > 1) {
            const float2 l = strat_2d(sp, ref, rng.pixel, rng.sample, rng.seed, 1);
            c.lx = l.x;
            c.ly = l.y;
        } else {
            float b[4];
            rng.block(0, b);
            c.lx = b[2];
            c.ly = b[3];
        }
    }
    return c;
}

// concentric_sample_disk (sampling.rs:181-198)
BG_D float2 concentric_sample_disk(float u0, float u1) {
    const float ox = 2.0f * u0 - 1.0f, oy = 2.0f * u1 - 1.0f;
    if (ox == 0.0f && oy == 0.0f) return make_float2(0.0f, 0.0f);
    float theta, r;
    if (fabsf(ox) > fabsf(oy)) {
        theta = (PI / 4.0f) * (oy / ox);
        r = ox;
    } else {
        theta = PI_OVER_TWO - (PI / 4.0f) * (ox / oy);
        r = oy;
    }
    return make_float2(r * cosf(theta), r * sinf(theta));
}
// The camera-space origin and direction of a thin-lens camera ray (perspective.rs:127-139): the
// lens point lens_radius * concentric_sample_disk(u) and the point where the pinhole direction d
// meets the plane of focus.
BG_D void thin_lens(const Camera& c, V3 d, float lu0, float lu1, V3* o, V3* dir) {
    const float2 l = concentric_sample_disk(lu0, lu1);
    const float lx = c.lens_radius * l.x, ly = c.lens_radius * l.y;
    const float t = c.focal_distance / d.z;
    const V3 focus = v3(0.0f + d.x * t, 0.0f + d.y * t, 0.0f + d.z * t);  // Ray::at from the origin
    *o = v3(lx, ly, 0.0f);
    *dir = normalize(focus - *o);
}
}  // namespace bg

// CPU ORACLE - TEST INFRASTRUCTURE ONLY.
//
// Plain C++17 restatement of the arithmetic helpers of kazijawad/bonsai (Rust, f32 build).
// Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use this code, as the test oracle.
// Parity unpinned: the reference ships no tests, golden vectors or fixtures for this path, and
// its Rust toolchain is absent, so this restatement cannot be checked against reference output.
//
// Semantics kept from the reference (compile with -ffp-contract=off, no fast-math):
//  * Vec3/Point3/Normal division by a scalar multiplies by the reciprocal
//    (src/geometries/vec3.rs:330-366, point3.rs:420-456, normal.rs:225-260).
//  * cross products are evaluated in f64 and rounded to f32 (src/geometries/vec3.rs:108-122).
//  * dot products sum left to right (src/geometries/vec3.rs:124-127).
//  * f32::min/max ignore a NaN operand (Rust semantics) -> fminf/fmaxf.
#pragma once
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>

namespace orc {

static const float PI = 3.14159265358979323846f;  // std::f32::consts::PI
static const float INV_PI = 1.0f / PI;            // src/base/constants.rs:13
static const float PI_OVER_TWO = PI / 2.0f;       // src/base/constants.rs:12
static const float MACHINE_EPSILON = FLT_EPSILON * 0.5f;        // constants.rs:16
static const float ONE_MINUS_EPSILON = 1.0f - FLT_EPSILON;      // constants.rs:15

// src/base/math.rs:3-5
inline float gamma(float n) { return (n * MACHINE_EPSILON) / (1.0f - n * MACHINE_EPSILON); }

inline uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// src/base/math.rs:11-25
inline float next_float_down(float v) {
    if (std::isinf(v) && v < 0.0f) return v;
    if (v == 0.0f) v = -0.0f;
    uint32_t ui = f2u(v);
    if (v > 0.0f) ui -= 1; else ui += 1;
    return u2f(ui);
}
// src/base/math.rs:27-41
inline float next_float_up(float v) {
    if (std::isinf(v) && v > 0.0f) return v;
    if (v == -0.0f) v = 0.0f;
    uint32_t ui = f2u(v);
    if (v >= 0.0f) ui += 1; else ui -= 1;
    return u2f(ui);
}

inline float rmin(float a, float b) { return std::fmin(a, b); }
inline float rmax(float a, float b) { return std::fmax(a, b); }
inline float rclamp(float v, float lo, float hi) {  // f32::clamp
    if (v < lo) v = lo;
    if (v > hi) v = hi;
    return v;
}

struct V3 {
    float x = 0, y = 0, z = 0;
    V3() = default;
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(V3 a, float s) { float inv = 1.0f / s; return {a.x * inv, a.y * inv, a.z * inv}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float abs_dot(V3 a, V3 b) { return std::fabs(dot(a, b)); }
inline V3 vabs(V3 a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }
inline float length_squared(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline float length(V3 a) { return std::sqrt(length_squared(a)); }
inline V3 normalize(V3 a) { return a / length(a); }
inline V3 cross(V3 a, V3 b) {  // src/geometries/vec3.rs:108-122
    double x = a.x, y = a.y, z = a.z, vx = b.x, vy = b.y, vz = b.z;
    return {(float)((y * vz) - (z * vy)), (float)((z * vx) - (x * vz)), (float)((x * vy) - (y * vx))};
}
inline float max_component(V3 a) { return rmax(a.x, rmax(a.y, a.z)); }
inline int max_dimension(V3 a) {  // src/geometries/vec3.rs:157-169
    if (a.x > a.y) return a.x > a.z ? 0 : 2;
    return a.y > a.z ? 1 : 2;
}
inline V3 permute(V3 a, int x, int y, int z) { return {a[x], a[y], a[z]}; }
inline V3 face_forward(V3 n, V3 v) { return dot(n, v) < 0.0f ? -n : n; }
inline float distance_squared(V3 a, V3 b) { return length_squared(a - b); }
inline float distance(V3 a, V3 b) { return length(a - b); }
// src/geometries/vec3.rs:25-33
inline void coordinate_system(V3 v1, V3* v2, V3* v3) {
    if (std::fabs(v1.x) > std::fabs(v1.y))
        *v2 = V3(-v1.z, 0.0f, v1.x) / std::sqrt(v1.x * v1.x + v1.z * v1.z);
    else
        *v2 = V3(0.0f, v1.z, -v1.y) / std::sqrt(v1.y * v1.y + v1.z * v1.z);
    *v3 = cross(v1, *v2);
}

// RGBSpectrum (src/spectra/rgb.rs): 3 x f32, componentwise ops, division by scalar via reciprocal.
struct RGB {
    float c[3] = {0, 0, 0};
    RGB() = default;
    explicit RGB(float v) { c[0] = c[1] = c[2] = v; }
    RGB(float r, float g, float b) { c[0] = r; c[1] = g; c[2] = b; }
    bool is_black() const { return c[0] == 0.0f && c[1] == 0.0f && c[2] == 0.0f; }
    bool is_nan() const { return std::isnan(c[0]) || std::isnan(c[1]) || std::isnan(c[2]); }
    float max_component_value() const { return rmax(rmax(c[0], c[1]), c[2]); }
    float y() const { return 0.212671f * c[0] + 0.715160f * c[1] + 0.072169f * c[2]; }  // rgb.rs:101-104
};
inline RGB operator+(RGB a, RGB b) { return {a.c[0] + b.c[0], a.c[1] + b.c[1], a.c[2] + b.c[2]}; }
inline RGB operator-(RGB a, RGB b) { return {a.c[0] - b.c[0], a.c[1] - b.c[1], a.c[2] - b.c[2]}; }
inline RGB operator*(RGB a, RGB b) { return {a.c[0] * b.c[0], a.c[1] * b.c[1], a.c[2] * b.c[2]}; }
inline RGB operator/(RGB a, RGB b) { return {a.c[0] / b.c[0], a.c[1] / b.c[1], a.c[2] / b.c[2]}; }
inline RGB operator*(RGB a, float s) { return {a.c[0] * s, a.c[1] * s, a.c[2] * s}; }
inline RGB operator*(float s, RGB a) { return {s * a.c[0], s * a.c[1], s * a.c[2]}; }
inline RGB operator/(RGB a, float s) { float inv = 1.0f / s; return {a.c[0] * inv, a.c[1] * inv, a.c[2] * inv}; }
inline RGB rgb_sqrt(RGB a) { return {std::sqrt(a.c[0]), std::sqrt(a.c[1]), std::sqrt(a.c[2])}; }

// EFloat (src/base/efloat.rs): running-error interval float.
struct EFloat {
    float v = 0, low = 0, high = 0;
    EFloat() = default;
    EFloat(float val, float err) {  // efloat.rs:18-34
        v = val;
        if (err == 0.0f) { low = high = val; }
        else { low = next_float_down(val - err); high = next_float_up(val + err); }
    }
    static EFloat raw(float v, float lo, float hi) { EFloat e; e.v = v; e.low = lo; e.high = hi; return e; }
};
inline EFloat operator+(EFloat a, EFloat b) {
    return EFloat::raw(a.v + b.v, next_float_down(a.low + b.low), next_float_up(a.high + b.high));
}
inline EFloat operator-(EFloat a, EFloat b) {
    return EFloat::raw(a.v - b.v, next_float_down(a.low - b.high), next_float_up(a.high - b.low));
}
inline EFloat operator*(EFloat a, EFloat b) {
    float p0 = a.low * b.low, p1 = a.high * b.low, p2 = a.low * b.high, p3 = a.high * b.high;
    return EFloat::raw(a.v * b.v, next_float_down(rmin(rmin(rmin(p0, p1), p2), p3)),
                       next_float_up(rmax(rmax(rmax(p0, p1), p2), p3)));
}
inline EFloat operator/(EFloat a, EFloat b) {
    float q0 = a.low / b.low, q1 = a.high / b.low, q2 = a.low / b.high, q3 = a.high / b.high;
    bool straddle = b.low < 0.0f && b.high > 0.0f;
    float lo = straddle ? -INFINITY : next_float_down(rmin(rmin(rmin(q0, q1), q2), q3));
    float hi = straddle ? INFINITY : next_float_up(rmax(rmax(rmax(q0, q1), q2), q3));
    return EFloat::raw(a.v / b.v, lo, hi);
}
inline EFloat operator-(EFloat a) { return EFloat::raw(-a.v, -a.high, -a.low); }
inline EFloat ef(float v) { return EFloat(v, 0.0f); }
// efloat.rs:36-67 (discriminant in f64)
inline bool quadratic(EFloat a, EFloat b, EFloat c, EFloat* t0, EFloat* t1) {
    double discrim = (double)b.v * (double)b.v - 4.0 * (double)a.v * (double)c.v;
    if (discrim < 0.0) return false;
    float root = (float)std::sqrt(discrim);
    EFloat rootf(root, MACHINE_EPSILON * root);
    EFloat q = (b.v < 0.0f) ? ef(-0.5f) * (b - rootf) : ef(-0.5f) * (b + rootf);
    *t0 = q / a;
    *t1 = c / q;
    if (t0->v > t1->v) { EFloat t = *t0; *t0 = *t1; *t1 = t; }
    return true;
}

// ---- counter-based RNG (Philox4x32-10, Salmon et al., SC'11), the same stream the device uses.
// key = {pixel index, low 32 bits of the seed}; counter = {sample index, dimension / 4,
// high 32 bits of the seed, 0x626F6E73}.  Lane = dimension % 4.  A uniform float keeps the
// top 23 bits, x = (u >> 9) * 2^-23, the value grid of rand 0.8's Uniform<f32>(0..1).
inline void philox4x32_10(uint32_t ctr[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * ctr[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * ctr[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ ctr[1] ^ k0, n2 = hi0 ^ ctr[3] ^ k1;
        ctr[0] = n0; ctr[1] = lo1; ctr[2] = n2; ctr[3] = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
}
struct CounterRng {
    uint32_t pixel = 0, sample = 0;
    uint64_t seed = 0;
    uint32_t stream = 0;  // the Whitted / direct-lighting integrators: node id - 1 of the ray tree
    float u(uint32_t dim) const {
        uint32_t ctr[4] = {sample, dim >> 2, (uint32_t)(seed >> 32), 0x626F6E73u ^ stream};
        philox4x32_10(ctr, pixel, (uint32_t)seed);
        uint32_t x = ctr[dim & 3];
        return (float)(x >> 9) * 0x1p-23f;
    }
    uint32_t bits(uint32_t dim) const {
        uint32_t ctr[4] = {sample, dim >> 2, (uint32_t)(seed >> 32), 0x626F6E73u ^ stream};
        philox4x32_10(ctr, pixel, (uint32_t)seed);
        return ctr[dim & 3];
    }
};

// StratifiedSampler (src/samplers/stratified.rs:75-137, src/base/sampling.rs:120-179) as the
// device draws it: a pixel's samples form passes of spp = nx * ny; stratified dimension k of sample
// s takes stratum perm_k(s % spp) (the identity under REF, F6: shuffle never swaps; a keyed
// permutation under PBRT), jittered by the counter RNG on stream 0x80000000 | 2k | is_2d (dimension
// 0 keys the permutation, 4 + 2j and 5 + 2j jitter stratum j).
struct Strat {
    uint32_t dims = 0, nx = 1, ny = 1, jitter = 0;
};
// The keyed bijection of [0, n) the device uses (cycle walking over a bijection of [0, 2^b)).
inline uint32_t strat_permute(uint32_t i, uint32_t n, uint32_t key) {
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
    return i;
}
inline uint32_t strat_stratum(const Strat& sp, bool ref, const CounterRng& rng, uint32_t k, uint32_t is2d,
                              CounterRng* jr) {
    const uint32_t n = sp.nx * sp.ny;
    *jr = CounterRng();
    jr->pixel = rng.pixel;
    jr->sample = rng.sample / n;
    jr->seed = rng.seed;
    jr->stream = 0x80000000u | (k << 1) | is2d;
    const uint32_t s = rng.sample % n;
    return ref ? s : strat_permute(s, n, jr->bits(0));
}
inline float strat_1d(const Strat& sp, bool ref, const CounterRng& rng, uint32_t k) {  // stratified_sample_1d
    CounterRng jr;
    const uint32_t j = strat_stratum(sp, ref, rng, k, 0u, &jr);
    const float delta = sp.jitter ? jr.u(4 + 2 * j) : 0.5f;
    const float inv = 1.0f / (float)(sp.nx * sp.ny);
    return std::fmin(((float)j + delta) * inv, ONE_MINUS_EPSILON);
}
inline void strat_2d(const Strat& sp, bool ref, const CounterRng& rng, uint32_t k, float* a, float* b) {
    CounterRng jr;
    const uint32_t j = strat_stratum(sp, ref, rng, k, 1u, &jr);
    const float jx = sp.jitter ? jr.u(4 + 2 * j) : 0.5f, jy = sp.jitter ? jr.u(5 + 2 * j) : 0.5f;
    const float dx = 1.0f / (float)sp.nx, dy = 1.0f / (float)sp.ny;
    *a = std::fmin(((float)(j % sp.nx) + jx) * dx, ONE_MINUS_EPSILON);
    *b = std::fmin(((float)(j / sp.nx) + jy) * dy, ONE_MINUS_EPSILON);
}
// Sampler::get_1d / get_2d of one sample in call order: stratified below sp.dims, else `v` (the
// counter RNG's value for the call's fixed dimension).
struct SamplerCalls {
    const Strat& sp;
    bool ref;
    const CounterRng& rng;
    uint32_t k1 = 0, k2 = 0;
    float get_1d(float v) {
        if (k1 < sp.dims) v = strat_1d(sp, ref, rng, k1);
        ++k1;
        return v;
    }
    void get_2d(float* a, float* b) {
        if (k2 < sp.dims) strat_2d(sp, ref, rng, k2, a, b);
        ++k2;
    }
};
// Dimension schedule (identical on the device): camera film.xy 0-1, lens 2-3, time 4;
// bounce b uses 8+8b: light pick, +1..2 u_light, +3..4 u_scattering, +5..6 BSDF, +7 roulette.
enum : uint32_t { DIM_FILM = 0, DIM_LENS = 2, DIM_TIME = 4, DIM_BOUNCE0 = 8, DIMS_PER_BOUNCE = 8 };
enum : uint32_t { BD_LIGHT = 0, BD_ULIGHT = 1, BD_USCAT = 3, BD_BSDF = 5, BD_RR = 7 };

}  // namespace orc

// CPU ORACLE - TEST INFRASTRUCTURE ONLY (the oracle of the tests, never the product path).
//
// C++17 restatement of the path-tracing hot path of kazijawad/bonsai (Rust, f32 build).
// Parity unpinned: the reference has no tests, golden vectors or fixtures for this path and its
// Rust toolchain is absent here, so this restatement could not be run against reference output.
// Every function names the reference file:line it follows.  Two estimator modes:
//   REF_COMPAT - the reference as written, defects included (F1..F14 in the design notes);
//   PBRT       - the same code with those defects fixed (PBRT-v3 PathIntegrator semantics).
// Random numbers come from the counter RNG in orc_core.hpp (the reference draws from ChaCha12
// seeded per 16x16 tile, src/base/integrator.rs:52-53; parity with it is statistical).
#include <algorithm>
#include <functional>
#include <atomic>
#include <mutex>
#include <thread>
#include <vector>

#include "../include/bonsai_gpu.h"
#include "orc_core.hpp"

namespace orc {

enum Mode { REF = 0, PBRT = 1 };

struct Ray {
    V3 o, d;
    float t_max = INFINITY;
    float time = 0.0f;
};

// ---------------------------------------------------------------- Mat4 / Transform
struct Mat4 {  // src/geometries/mat4.rs
    float m[4][4];
    static Mat4 identity() {
        Mat4 r;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) r.m[i][j] = (i == j) ? 1.0f : 0.0f;
        return r;
    }
};
static Mat4 mat_mul(const Mat4& a, const Mat4& b) {  // mat4.rs:36-48
    Mat4 r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j] +
                        a.m[i][3] * b.m[3][j];
    return r;
}
static Mat4 mat_inverse(const Mat4& in) {  // mat4.rs:72-140 (Gauss-Jordan, full pivoting)
    float minv[4][4];
    std::memcpy(minv, in.m, sizeof(minv));
    int ic[4] = {0}, ir[4] = {0}, piv[4] = {0};
    for (int i = 0; i < 4; ++i) {
        int row = 0, col = 0;
        float big = 0.0f;
        for (int j = 0; j < 4; ++j) {
            if (piv[j] != 1) {
                for (int k = 0; k < 4; ++k) {
                    if (piv[k] == 0) {
                        if (std::fabs(minv[j][k]) >= big) {
                            big = std::fabs(minv[j][k]);
                            row = j;
                            col = k;
                        }
                    }
                }
            }
        }
        piv[col] += 1;
        if (row != col)
            for (int k = 0; k < 4; ++k) std::swap(minv[row][k], minv[col][k]);
        ir[i] = row;
        ic[i] = col;
        float pinv = 1.0f / minv[col][col];
        minv[col][col] = 1.0f;
        for (int j = 0; j < 4; ++j) minv[col][j] *= pinv;
        for (int j = 0; j < 4; ++j) {
            if (j != col) {
                float save = minv[j][col];
                minv[j][col] = 0.0f;
                for (int k = 0; k < 4; ++k) minv[j][k] -= minv[col][k] * save;
            }
        }
    }
    for (int j = 3; j >= 0; --j)
        if (ir[j] != ic[j])
            for (int k = 0; k < 4; ++k) std::swap(minv[k][ir[j]], minv[k][ic[j]]);
    Mat4 r;
    std::memcpy(r.m, minv, sizeof(minv));
    return r;
}
struct Transform {
    Mat4 m, mi;
};
static Transform t_mul(const Transform& a, const Transform& b) {  // transform.rs:1629-1649
    return {mat_mul(a.m, b.m), mat_mul(b.mi, a.mi)};
}
static Transform t_inverse(const Transform& t) { return {t.mi, t.m}; }
static Transform t_scale(float x, float y, float z) {  // transform.rs:118-150
    Transform t{Mat4::identity(), Mat4::identity()};
    t.m.m[0][0] = x; t.m.m[1][1] = y; t.m.m[2][2] = z;
    t.mi.m[0][0] = 1.0f / x; t.mi.m[1][1] = 1.0f / y; t.mi.m[2][2] = 1.0f / z;
    return t;
}
static Transform t_translate(V3 d) {  // transform.rs:88-98
    Transform t{Mat4::identity(), Mat4::identity()};
    t.m.m[0][3] = d.x; t.m.m[1][3] = d.y; t.m.m[2][3] = d.z;
    t.mi.m[0][3] = -d.x; t.mi.m[1][3] = -d.y; t.mi.m[2][3] = -d.z;
    return t;
}
static bool is_identity(const Transform& t) {
    Mat4 id = Mat4::identity();
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            if (t.m.m[i][j] != id.m[i][j]) return false;
    return true;
}
static Transform t_perspective(float fov, float n, float f) {  // transform.rs:48-73
    Mat4 mat = Mat4::identity();
    mat.m[2][2] = f / (f - n);
    mat.m[2][3] = -f * n / (f - n);
    mat.m[3][2] = 1.0f;
    mat.m[3][3] = 0.0f;
    Mat4 inv = mat_inverse(mat);
    float rad = fov * (PI / 180.0f);
    float inv_tan = 1.0f / std::tan(rad / 2.0f);
    return t_mul(t_scale(inv_tan, inv_tan, 1.0f), Transform{mat, inv});
}
static Transform t_look_at(V3 pos, V3 look, V3 up) {  // transform.rs:152-189 (camera_to_world)
    Mat4 c2w = Mat4::identity();
    c2w.m[0][3] = pos.x; c2w.m[1][3] = pos.y; c2w.m[2][3] = pos.z; c2w.m[3][3] = 1.0f;
    V3 dir = normalize(look - pos);
    if (length(cross(normalize(up), dir)) == 0.0f) return {Mat4::identity(), Mat4::identity()};
    V3 right = normalize(cross(normalize(up), dir));
    V3 new_up = cross(dir, right);
    c2w.m[0][0] = right.x; c2w.m[1][0] = right.y; c2w.m[2][0] = right.z; c2w.m[3][0] = 0.0f;
    c2w.m[0][1] = new_up.x; c2w.m[1][1] = new_up.y; c2w.m[2][1] = new_up.z; c2w.m[3][1] = 0.0f;
    c2w.m[0][2] = dir.x; c2w.m[1][2] = dir.y; c2w.m[2][2] = dir.z; c2w.m[3][2] = 0.0f;
    return {c2w, mat_inverse(c2w)};
}
static V3 xf_point(const Transform& t, V3 p) {  // point3.rs:51-69
    const auto& m = t.m.m;
    float xp = m[0][0] * p.x + m[0][1] * p.y + m[0][2] * p.z + m[0][3];
    float yp = m[1][0] * p.x + m[1][1] * p.y + m[1][2] * p.z + m[1][3];
    float zp = m[2][0] * p.x + m[2][1] * p.y + m[2][2] * p.z + m[2][3];
    float wp = m[3][0] * p.x + m[3][1] * p.y + m[3][2] * p.z + m[3][3];
    if (wp == 1.0f) return {xp, yp, zp};
    return V3(xp, yp, zp) / wp;
}
static V3 xf_point_err(const Transform& t, V3 p, V3* err) {  // point3.rs:71-100
    const auto& m = t.m.m;
    float x = p.x, y = p.y, z = p.z;
    float xp = (m[0][0] * x + m[0][1] * y) + (m[0][2] * z + m[0][3]);
    float yp = (m[1][0] * x + m[1][1] * y) + (m[1][2] * z + m[1][3]);
    float zp = (m[2][0] * x + m[2][1] * y) + (m[2][2] * z + m[2][3]);
    float wp = (m[3][0] * x + m[3][1] * y) + (m[3][2] * z + m[3][3]);
    float xa = std::fabs(m[0][0] * x) + std::fabs(m[0][1] * y) + std::fabs(m[0][2] * z) + std::fabs(m[0][3]);
    float ya = std::fabs(m[1][0] * x) + std::fabs(m[1][1] * y) + std::fabs(m[1][2] * z) + std::fabs(m[1][3]);
    float za = std::fabs(m[2][0] * x) + std::fabs(m[2][1] * y) + std::fabs(m[2][2] * z) + std::fabs(m[2][3]);
    *err = gamma(3.0f) * V3(xa, ya, za);
    if (wp == 1.0f) return {xp, yp, zp};
    return V3(xp, yp, zp) / wp;
}
static V3 xf_point_perr(const Transform& t, V3 p, V3 pe, V3* abs_err) {  // point3.rs:102-140
    const auto& m = t.m.m;
    float x = p.x, y = p.y, z = p.z;
    float xp = (m[0][0] * x + m[0][1] * y) + (m[0][2] * z + m[0][3]);
    float yp = (m[1][0] * x + m[1][1] * y) + (m[1][2] * z + m[1][3]);
    float zp = (m[2][0] * x + m[2][1] * y) + (m[2][2] * z + m[2][3]);
    float wp = (m[3][0] * x + m[3][1] * y) + (m[3][2] * z + m[3][3]);
    float g3 = gamma(3.0f);
    for (int i = 0; i < 3; ++i) {
        (*abs_err)[i] = (g3 + 1.0f) * (std::fabs(m[i][0]) * pe.x + std::fabs(m[i][1]) * pe.y +
                                       std::fabs(m[i][2]) * pe.z) +
                        g3 * (std::fabs(m[i][0] * x) + std::fabs(m[i][1] * y) +
                              std::fabs(m[i][2] * z) + std::fabs(m[i][3]));
    }
    if (wp == 1.0f) return {xp, yp, zp};
    return V3(xp, yp, zp) / wp;
}
static V3 xf_vec(const Transform& t, V3 v) {  // vec3.rs:35-44
    const auto& m = t.m.m;
    return {m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z, m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z,
            m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z};
}
static V3 xf_vec_err(const Transform& t, V3 v, V3* e) {  // vec3.rs:46-64
    const auto& m = t.m.m;
    float g3 = gamma(3.0f);
    e->x = g3 * (std::fabs(m[0][0] * v.x) + std::fabs(m[0][1] * v.y) + std::fabs(m[0][2] * v.z));
    e->y = g3 * (std::fabs(m[1][0] * v.x) + std::fabs(m[1][1] * v.y) + std::fabs(m[1][2] * v.z));
    e->z = g3 * (std::fabs(m[2][0] * v.x) + std::fabs(m[2][1] * v.y) + std::fabs(m[2][2] * v.z));
    return xf_vec(t, v);
}
static V3 xf_normal(const Transform& t, V3 n) {  // normal.rs:21-30
    const auto& mi = t.mi.m;
    return {mi[0][0] * n.x + mi[1][0] * n.y + mi[2][0] * n.z, mi[0][1] * n.x + mi[1][1] * n.y + mi[2][1] * n.z,
            mi[0][2] * n.x + mi[1][2] * n.y + mi[2][2] * n.z};
}
static Ray xf_ray(const Transform& t, const Ray& r) {  // ray.rs:50-76
    V3 oerr;
    V3 o = xf_point_err(t, r.o, &oerr);
    V3 d = xf_vec(t, r.d);
    float ls = length_squared(d);
    float t_max = r.t_max;
    if (ls > 0.0f) {
        float dt = dot(vabs(d), oerr) / ls;
        o = o + d * dt;
        t_max -= dt;
    }
    return {o, d, t_max, r.time};
}
static Ray xf_ray_err(const Transform& t, const Ray& r, V3* oe, V3* de) {  // ray.rs:78-106
    V3 o = xf_point_err(t, r.o, oe);
    V3 d = xf_vec_err(t, r.d, de);
    float ls = length_squared(d);
    if (ls > 0.0f) {
        float dt = dot(vabs(d), *oe) / ls;
        o = o + d * dt;
    }
    return {o, d, r.t_max, r.time};
}

// ---------------------------------------------------------------- Bounds3
struct Bounds3 {  // src/geometries/bounds3.rs; Default = (MAX, MIN) (bounds3.rs:291-298)
    V3 mn{FLT_MAX, FLT_MAX, FLT_MAX};
    V3 mx{-FLT_MAX, -FLT_MAX, -FLT_MAX};
    const V3& operator[](int i) const { return i == 0 ? mn : mx; }
    void unite(const Bounds3& b) {
        mn = {rmin(mn.x, b.mn.x), rmin(mn.y, b.mn.y), rmin(mn.z, b.mn.z)};
        mx = {rmax(mx.x, b.mx.x), rmax(mx.y, b.mx.y), rmax(mx.z, b.mx.z)};
    }
    void unite(V3 p) {
        mn = {rmin(mn.x, p.x), rmin(mn.y, p.y), rmin(mn.z, p.z)};
        mx = {rmax(mx.x, p.x), rmax(mx.y, p.y), rmax(mx.z, p.z)};
    }
    float surface_area() const {  // bounds3.rs:160-163
        V3 d = mx - mn;
        return 2.0f * (d.x * d.y + d.x * d.z + d.y * d.z);
    }
    int maximum_extent() const {  // bounds3.rs:175-184
        V3 d = mx - mn;
        if (d.x > d.y && d.x > d.z) return 0;
        if (d.y > d.z) return 1;
        return 2;
    }
    V3 offset(V3 p) const {  // bounds3.rs:194-206
        V3 o = p - mn;
        if (mx.x > mn.x) o.x /= mx.x - mn.x;
        if (mx.y > mn.y) o.y /= mx.y - mn.y;
        if (mx.z > mn.z) o.z /= mx.z - mn.z;
        return o;
    }
    // bounds3.rs:246-288
    bool intersect_p(const Ray& ray, V3 inv, const int neg[3]) const {
        float k = 1.0f + 2.0f * gamma(3.0f);
        float t_min = ((*this)[neg[0]].x - ray.o.x) * inv.x;
        float t_max = ((*this)[1 - neg[0]].x - ray.o.x) * inv.x;
        float ty_min = ((*this)[neg[1]].y - ray.o.y) * inv.y;
        float ty_max = ((*this)[1 - neg[1]].y - ray.o.y) * inv.y;
        t_max *= k;
        ty_max *= k;
        if (t_min > ty_max || ty_min > t_max) return false;
        if (ty_min > t_min) t_min = ty_min;
        if (ty_max < t_max) t_max = ty_max;
        float tz_min = ((*this)[neg[2]].z - ray.o.z) * inv.z;
        float tz_max = ((*this)[1 - neg[2]].z - ray.o.z) * inv.z;
        tz_max *= k;
        if (t_min > tz_max || tz_min > t_max) return false;
        if (tz_min > t_min) t_min = tz_min;
        if (tz_max < t_max) t_max = tz_max;
        return (t_min < ray.t_max) && (t_max > 0.0f);
    }
};

// ---------------------------------------------------------------- Interaction
struct Interaction {  // src/base/interaction.rs:47-54 (+ the SurfaceInteraction fields used)
    V3 p, p_err, wo, n;
    float time = 0.0f;
    bool surface = false;
    V3 dpdu, shading_n, shading_dpdu;
    int prim = -1;
    // SurfaceInteraction parameterisation (interaction.rs:18-45)
    float uv[2] = {0.0f, 0.0f};
    V3 dpdv, dndu, dndv, shading_dndu, shading_dndv;
    V3 dpdx, dpdy;
    float dudx = 0.0f, dvdx = 0.0f, dudy = 0.0f, dvdy = 0.0f;
};
// src/geometries/point3.rs:31-49
static V3 offset_ray_origin(V3 p, V3 perr, V3 n, V3 w) {
    V3 offset = dot(vabs(n), perr) * n;
    if (dot(w, n) < 0.0f) offset = -offset;
    V3 po = p + offset;
    for (int i = 0; i < 3; ++i) {
        if (offset[i] > 0.0f) po[i] = next_float_up(po[i]);
        else if (offset[i] < 0.0f) po[i] = next_float_down(po[i]);
    }
    return po;
}
// interaction.rs:115-121; F3: t_max = 1 - 0.0001 for a normalized direction (PBRT: infinity)
static Ray spawn_ray(const Interaction& it, V3 d, Mode mode) {
    V3 o = offset_ray_origin(it.p, it.p_err, it.n, d);
    return {o, d, mode == REF ? (1.0f - 0.0001f) : INFINITY, it.time};
}
// interaction.rs:132-143
static Ray spawn_ray_to_it(const Interaction& a, const Interaction& b) {
    V3 o = offset_ray_origin(a.p, a.p_err, a.n, b.p - a.p);
    V3 target = offset_ray_origin(b.p, b.p_err, b.n, o - b.p);
    return {o, target - o, 1.0f - 0.0001f, a.time};
}

// ---------------------------------------------------------------- Scene data
struct Sphere {  // src/shapes/sphere.rs:38-64 (translation-only object_to_world)
    Transform o2w, w2o;
    float radius, z_min, z_max, theta_min, theta_max, phi_max;
    uint32_t mat;
};
// Cylinder / Disk / Cone (src/shapes/{cylinder,disk,cone}.rs) with an affine transform.
struct Quadric {
    int kind;  // 0 cylinder, 1 disk, 2 cone
    Transform o2w, w2o;
    bool reverse, swaps;
    float radius, inner, z_min, z_max, height, phi_max;
    uint32_t mat;
};
enum : uint8_t { TA_REVERSE = 1, TA_SWAPS = 2, TA_NORMALS = 4 };
// ImageTexture / UVTexture + TextureMapping2D (src/textures/{image,uv}.rs, src/base/texture.rs)
// with the MIPMap pyramid (src/base/mipmap.rs, src/io/image.rs:55-159).
struct Image {
    int w = 0, h = 0;
    std::vector<float> px;  // Image::pixels, 3 per texel
};
struct Texture {
    uint32_t kind = 0, wrap = 0, mapping = 0;
    float su = 1, sv = 1, du = 0, dv = 0;
    Transform w2t;
    V3 vs, vt;
    float ds = 0, dt = 0;
    std::vector<Image> pyramid;
};
// InfiniteAreaLight (src/lights/infinite.rs:21-29) and its Distribution2D (sampling.rs:16-19)
struct InfiniteLight {
    Texture map;  // MIPMap of the scaled image, repeat wrap
    Transform l2w, w2l;
    V3 center;
    float radius = 0.0f;
    uint32_t nu = 0, nv = 0;
    std::vector<float> func;      // nv rows of nu; conditional v's function is the tail from v * nu
    std::vector<float> cond_cdf;  // nv rows of nu + 1
    std::vector<float> cond_int;  // per-row integrals: the marginal's function
    std::vector<float> marg_cdf;  // nv + 1
    float marg_int = 0.0f;
};
constexpr int64_t LIGHT_INF = -1;  // the infinite light's entry in Scene::light_prims
struct Scene {
    std::vector<V3> pos;  // 3 per triangle (TriangleMesh::position, triangle.rs:17-22)
    int64_t ntri = 0, nsph = 0, nquad = 0;
    std::vector<Quadric> quads;
    std::vector<uint32_t> tri_mat;
    std::vector<int32_t> prim_emission;  // emission record per primitive or -1
    std::vector<int32_t> prim_light;     // light-list index per primitive or -1
    std::vector<Sphere> sph;
    std::vector<bg_material> mats;
    std::vector<bg_area_light> emis;
    std::vector<int64_t> light_prims;  // Scene::lights (one DiffuseAreaLight per emitting shape)
    // TriangleMesh vertex attributes (triangle.rs:17-22) and TriangleOptions flags, per triangle
    std::vector<V3> tri_n;             // 3 per triangle (meaningful where TA_NORMALS is set)
    std::vector<float> tri_uv;         // 6 per triangle; empty: Triangle::get_uvs defaults
    std::vector<uint8_t> tri_flags;    // TA_* bits; empty: none
    std::vector<struct Texture> tex;
    bool has_inf = false;
    InfiniteLight inf;
    // BVH (src/accelerators/bvh.rs:20-31)
    struct Node {
        Bounds3 b;
        uint32_t offset = 0;  // primitive_offset (leaf) or second_child_offset (interior)
        uint32_t count = 0;
        uint32_t axis = 0;
    };
    std::vector<Node> nodes;
    std::vector<uint32_t> order;  // ordered_primitives
    int64_t nprims() const { return ntri + nsph + nquad; }
};

struct Counters {
    int64_t ext_rays = 0, shadow_rays = 0, ext_visits = 0, ext_tests = 0, sh_visits = 0, sh_tests = 0;
    int64_t nan_samples = 0;
    void add(const Counters& o) {
        ext_rays += o.ext_rays; shadow_rays += o.shadow_rays; ext_visits += o.ext_visits;
        ext_tests += o.ext_tests; sh_visits += o.sh_visits; sh_tests += o.sh_tests;
        nan_samples += o.nan_samples;
    }
};

// ---------------------------------------------------------------- Triangle (triangle.rs)
static bool tri_intersect(const Scene& s, int64_t i, const Ray& ray, float* t_hit, Interaction* it,
                          bool test_only) {
    const V3& p0 = s.pos[3 * i];
    const V3& p1 = s.pos[3 * i + 1];
    const V3& p2 = s.pos[3 * i + 2];
    V3 p0t = p0 - ray.o, p1t = p1 - ray.o, p2t = p2 - ray.o;  // :141-145
    int kz = max_dimension(vabs(ray.d));                      // :147-156
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    V3 d = permute(ray.d, kx, ky, kz);
    p0t = permute(p0t, kx, ky, kz);
    p1t = permute(p1t, kx, ky, kz);
    p2t = permute(p2t, kx, ky, kz);
    float sx = -d.x / d.z, sy = -d.y / d.z, sz = 1.0f / d.z;  // :162-171
    p0t.x += sx * p0t.z; p0t.y += sy * p0t.z;
    p1t.x += sx * p1t.z; p1t.y += sy * p1t.z;
    p2t.x += sx * p2t.z; p2t.y += sy * p2t.z;
    float e0 = p1t.x * p2t.y - p1t.y * p2t.x;  // :173-176
    float e1 = p2t.x * p0t.y - p2t.y * p0t.x;
    float e2 = p0t.x * p1t.y - p0t.y * p1t.x;
    if (e0 == 0.0f || e1 == 0.0f || e2 == 0.0f) {  // :178-190 f64 fallback
        double a = (double)p2t.x * (double)p1t.y, b = (double)p2t.y * (double)p1t.x;
        e0 = (float)(b - a);
        double c = (double)p0t.x * (double)p2t.y, dd = (double)p0t.y * (double)p2t.x;
        e1 = (float)(dd - c);
        double e = (double)p1t.x * (double)p0t.y, f = (double)p1t.y * (double)p0t.x;
        e2 = (float)(f - e);
    }
    if ((e0 < 0.0f || e1 < 0.0f || e2 < 0.0f) && (e0 > 0.0f || e1 > 0.0f || e2 > 0.0f)) return false;
    float det = e0 + e1 + e2;
    if (det == 0.0f) return false;
    p0t.z *= sz; p1t.z *= sz; p2t.z *= sz;  // :201-210
    float t_scaled = e0 * p0t.z + e1 * p1t.z + e2 * p2t.z;
    if (det < 0.0f && (t_scaled >= 0.0f || t_scaled < ray.t_max * det)) return false;
    else if (det > 0.0f && (t_scaled <= 0.0f || t_scaled > ray.t_max * det)) return false;
    float inv_det = 1.0f / det;  // :212-217
    float b0 = e0 * inv_det, b1 = e1 * inv_det, b2 = e2 * inv_det;
    float t = t_scaled * inv_det;
    float max_zt = max_component(vabs(V3(p0t.z, p1t.z, p2t.z)));  // :219-239
    float delta_z = gamma(3.0f) * max_zt;
    float max_xt = max_component(vabs(V3(p0t.x, p1t.x, p2t.x)));
    float max_yt = max_component(vabs(V3(p0t.y, p1t.y, p2t.y)));
    float delta_x = gamma(5.0f) * (max_xt + max_zt);
    float delta_y = gamma(5.0f) * (max_yt + max_zt);
    float delta_e = 2.0f * (gamma(2.0f) * max_xt * max_yt + delta_y * max_xt + delta_x * max_yt);
    float max_e = max_component(vabs(V3(e0, e1, e2)));
    float delta_t = 3.0f * (gamma(3.0f) * max_e * max_zt + delta_e * max_zt + delta_z * max_e) *
                    std::fabs(inv_det);
    if (t <= delta_t) return false;
    // uvs (Triangle::get_uvs, :107-117) and partial derivatives (:241-268)
    float uv[3][2] = {{0.0f, 0.0f}, {1.0f, 0.0f}, {1.0f, 1.0f}};
    if (!s.tri_uv.empty())
        for (int k = 0; k < 3; ++k) {
            uv[k][0] = s.tri_uv[6 * i + 2 * k];
            uv[k][1] = s.tri_uv[6 * i + 2 * k + 1];
        }
    float duv02[2] = {uv[0][0] - uv[2][0], uv[0][1] - uv[2][1]};
    float duv12[2] = {uv[1][0] - uv[2][0], uv[1][1] - uv[2][1]};
    V3 dp02 = p0 - p2, dp12 = p1 - p2;
    float uvdet = duv02[0] * duv12[1] - duv02[1] * duv12[0];
    bool degenerate_uv = std::fabs(uvdet) < 1e-8f;
    V3 dpdu, dpdv;
    if (!degenerate_uv) {
        float invd = 1.0f / uvdet;
        dpdu = (duv12[1] * dp02 - duv02[1] * dp12) * invd;
        dpdv = (-duv12[0] * dp02 + duv02[0] * dp12) * invd;
    }
    if (degenerate_uv || length_squared(cross(dpdu, dpdv)) == 0.0f) {
        V3 ng = cross(p2 - p0, p1 - p0);
        if (length_squared(ng) == 0.0f) return false;
        coordinate_system(normalize(ng), &dpdu, &dpdv);
    }
    if (test_only) return true;
    const uint8_t fl = s.tri_flags.empty() ? 0 : s.tri_flags[i];
    const bool reverse = (fl & TA_REVERSE) != 0, swaps = (fl & TA_SWAPS) != 0;
    // error bounds, hit point and uv (:270-278)
    float xs = std::fabs(b0 * p0.x) + std::fabs(b1 * p1.x) + std::fabs(b2 * p2.x);
    float ys = std::fabs(b0 * p0.y) + std::fabs(b1 * p1.y) + std::fabs(b2 * p2.y);
    float zs = std::fabs(b0 * p0.z) + std::fabs(b1 * p1.z) + std::fabs(b2 * p2.z);
    V3 perr = gamma(7.0f) * V3(xs, ys, zs);
    V3 phit = b0 * p0 + b1 * p1 + b2 * p2;
    // Interaction::new (interaction.rs:57-100): shading geometry starts as the true geometry
    it->p = phit;
    it->p_err = perr;
    it->time = ray.time;
    it->wo = -ray.d;
    it->surface = true;
    it->uv[0] = b0 * uv[0][0] + b1 * uv[1][0] + b2 * uv[2][0];
    it->uv[1] = b0 * uv[0][1] + b1 * uv[1][1] + b2 * uv[2][1];
    it->dpdu = dpdu;
    it->dpdv = dpdv;
    it->dndu = it->dndv = V3(0, 0, 0);
    it->shading_dpdu = dpdu;
    it->shading_dndu = it->shading_dndv = V3(0, 0, 0);
    // the normal is overridden with the winding normal (:299-307)
    V3 nn = normalize(cross(dp02, dp12));
    if (reverse ^ swaps) nn = -nn;
    it->n = nn;
    it->shading_n = nn;
    if (fl & TA_NORMALS) {  // shading geometry from the vertex normals (:309-398)
        const V3 n0 = s.tri_n[3 * i], n1 = s.tri_n[3 * i + 1], n2 = s.tri_n[3 * i + 2];
        V3 sn = b0 * n0 + b1 * n1 + b2 * n2;
        sn = length_squared(sn) > 0.0f ? normalize(sn) : it->n;
        V3 st = normalize(it->dpdu);
        V3 sb = cross(st, sn);
        if (length_squared(sb) > 0.0f) {
            sb = normalize(sb);
            st = cross(sb, sn);
        } else {
            coordinate_system(sn, &st, &sb);
        }
        V3 dndu(0, 0, 0), dndv(0, 0, 0);
        V3 dn1 = n0 - n2, dn2 = n1 - n2;
        if (degenerate_uv) {
            V3 dn = cross(n2 - n0, n1 - n0);
            if (length_squared(dn) != 0.0f) coordinate_system(dn, &dndu, &dndv);
        } else {
            float invd = 1.0f / uvdet;
            dndu = (duv12[1] * dn1 - duv02[1] * dn2) * invd;
            dndv = (-duv12[0] * dn1 + duv02[0] * dn2) * invd;
        }
        if (reverse) sb = -sb;
        // Interaction::set_shading_geometry(st, sb, dndu, dndv, true) (interaction.rs:145-168)
        it->shading_n = normalize(cross(st, sb));
        it->n = face_forward(it->n, it->shading_n);
        it->shading_dpdu = st;
        it->shading_dndu = dndu;
        it->shading_dndv = dndv;
    }
    *t_hit = t;
    return true;
}
static float tri_area(const Scene& s, int64_t i) {  // triangle.rs:561-566
    const V3& p0 = s.pos[3 * i];
    return 0.5f * length(cross(s.pos[3 * i + 1] - p0, s.pos[3 * i + 2] - p0));
}
static Interaction tri_sample(const Scene& s, int64_t i, float u0, float u1, float* pdf) {  // :522-559
    float sq = std::sqrt(u0);  // uniform_sample_triangle (sampling.rs:233-236)
    float b0 = 1.0f - sq, b1 = u1 * sq;
    const V3& p0 = s.pos[3 * i];
    const V3& p1 = s.pos[3 * i + 1];
    const V3& p2 = s.pos[3 * i + 2];
    float b2 = 1.0f - b0 - b1;
    Interaction r;
    r.p = b0 * p0 + b1 * p1 + b2 * p2;
    r.n = normalize(cross(p1 - p0, p2 - p0));
    const uint8_t fl = s.tri_flags.empty() ? 0 : s.tri_flags[i];
    if (fl & TA_NORMALS) {  // face the interpolated vertex normal (:534-545)
        V3 shaded = b0 * s.tri_n[3 * i] + b1 * s.tri_n[3 * i + 1] + (1.0f - b0 - b1) * s.tri_n[3 * i + 2];
        r.n = face_forward(r.n, shaded);
    } else if (((fl & TA_REVERSE) != 0) ^ ((fl & TA_SWAPS) != 0)) {
        r.n = r.n * -1.0f;
    }
    V3 pabs = vabs(b0 * p0) + vabs(b1 * p1) + vabs(b2 * p2);
    r.p_err = gamma(6.0f) * pabs;
    *pdf = 1.0f / tri_area(s, i);
    return r;
}

// Weingarten equations (sphere.rs:191-204; the same in cylinder.rs and cone.rs)
static void fundamental_forms(V3 dpdu, V3 dpdv, V3 d2pduu, V3 d2pduv, V3 d2pdvv, V3* dndu, V3* dndv) {
    float E = dot(dpdu, dpdu), F = dot(dpdu, dpdv), G = dot(dpdv, dpdv);
    V3 N = normalize(cross(dpdu, dpdv));
    float e = dot(N, d2pduu), f = dot(N, d2pduv), g = dot(N, d2pdvv);
    float inv = 1.0f / (E * G - F * F);
    *dndu = (f * F - e * G) * inv * dpdu + (e * F - f * E) * inv * dpdv;
    *dndv = (g * F - f * G) * inv * dpdu + (f * F - g * E) * inv * dpdv;
}

// ---------------------------------------------------------------- Sphere (sphere.rs)
static bool sphere_intersect(const Sphere& sp, const Ray& r_world, float* t_hit, Interaction* it,
                             bool test_only) {
    V3 oe, de;
    Ray ray = xf_ray_err(sp.w2o, r_world, &oe, &de);  // :80-83
    EFloat ox(ray.o.x, oe.x), oy(ray.o.y, oe.y), oz(ray.o.z, oe.z);
    EFloat dx(ray.d.x, de.x), dy(ray.d.y, de.y), dz(ray.d.z, de.z);
    EFloat a = dx * dx + dy * dy + dz * dz;
    EFloat b = ef(2.0f) * (dx * ox + dy * oy + dz * oz);
    EFloat c = ox * ox + oy * oy + oz * oz - ef(sp.radius) * ef(sp.radius);
    EFloat t0, t1;
    if (!quadratic(a, b, c, &t0, &t1)) return false;
    if (t0.high > ray.t_max || t1.low <= 0.0f) return false;  // :106-116
    EFloat tsh = t0;
    if (tsh.low <= 0.0f) {
        tsh = t1;
        if (tsh.high > ray.t_max) return false;
    }
    auto refine = [&](float t) {
        V3 ph = ray.o + ray.d * t;
        ph = ph * (sp.radius / distance(ph, V3(0, 0, 0)));
        if (ph.x == 0.0f && ph.y == 0.0f) ph.x = 1e-5f * sp.radius;
        return ph;
    };
    V3 ph = refine(tsh.v);
    float phi = std::atan2(ph.y, ph.x);
    if (phi < 0.0f) phi += 2.0f * PI;
    auto clipped = [&](V3 p, float ph_) {
        return (sp.z_min > -sp.radius && p.z < sp.z_min) || (sp.z_max < sp.radius && p.z > sp.z_max) ||
               ph_ > sp.phi_max;
    };
    if (clipped(ph, phi)) {  // :127-161
        if (tsh.v == t1.v && tsh.low == t1.low && tsh.high == t1.high) return false;
        if (t1.high > ray.t_max) return false;
        tsh = t1;
        ph = refine(tsh.v);
        phi = std::atan2(ph.y, ph.x);
        if (phi < 0.0f) phi += 2.0f * PI;
        if (clipped(ph, phi)) return false;
    }
    if (test_only) return true;
    // parametric representation and partial derivatives (:163-176)
    float theta = std::acos(rclamp(ph.z / sp.radius, -1.0f, 1.0f));
    float z_radius = std::sqrt(ph.x * ph.x + ph.y * ph.y);
    float inv_zr = 1.0f / z_radius;
    float cos_phi = ph.x * inv_zr, sin_phi = ph.y * inv_zr;
    V3 dpdu(-sp.phi_max * ph.y, sp.phi_max * ph.x, 0.0f);
    V3 dpdv = (sp.theta_max - sp.theta_min) * V3(ph.z * cos_phi, ph.z * sin_phi, -sp.radius * std::sin(theta));
    // normal derivatives from the fundamental forms (:178-204)
    V3 d2pduu = -sp.phi_max * sp.phi_max * V3(ph.x, ph.y, 0.0f);
    V3 d2pduv = (sp.theta_max - sp.theta_min) * ph.z * sp.phi_max * V3(-sin_phi, cos_phi, 0.0f);
    V3 d2pdvv = -(sp.theta_max - sp.theta_min) * (sp.theta_max - sp.theta_min) * ph;
    V3 dndu, dndv;
    fundamental_forms(dpdu, dpdv, d2pduu, d2pduv, d2pdvv, &dndu, &dndv);
    V3 perr = gamma(5.0f) * vabs(ph);  // :209
    // Interaction::new then Interaction::transform(object_to_world) (interaction.rs:268-300)
    V3 n = normalize(cross(dpdu, dpdv));
    V3 abs_err;
    it->p = xf_point_perr(sp.o2w, ph, perr, &abs_err);
    it->p_err = abs_err;
    it->time = ray.time;
    it->wo = xf_vec(sp.o2w, -ray.d);
    it->n = normalize(xf_normal(sp.o2w, n));
    it->surface = true;
    it->uv[0] = phi / sp.phi_max;
    it->uv[1] = (theta - sp.theta_min) / (sp.theta_max - sp.theta_min);
    it->dpdu = xf_vec(sp.o2w, dpdu);
    it->dpdv = xf_vec(sp.o2w, dpdv);
    it->dndu = xf_normal(sp.o2w, dndu);
    it->dndv = xf_normal(sp.o2w, dndv);
    it->shading_n = face_forward(normalize(xf_normal(sp.o2w, n)), it->n);
    it->shading_dpdu = xf_vec(sp.o2w, dpdu);
    it->shading_dndu = it->dndu;
    it->shading_dndv = it->dndv;
    *t_hit = tsh.v;
    return true;
}

// ---------------------------------------------------------------- quadrics
inline float absolute_error(const EFloat& e) {  // efloat.rs absolute_error
    return next_float_up(rmax(std::fabs(e.high - e.v), std::fabs(e.v - e.low)));
}
// Interaction::new (interaction.rs:57-100) + Interaction::transform (interaction.rs:268-300)
static void quadric_interaction(const Quadric& q, V3 ph, V3 perr, const Ray& ray, V3 dpdu, V3 dpdv, float u,
                                float v, V3 dndu, V3 dndv, Interaction* it) {
    V3 n = normalize(cross(dpdu, dpdv));
    if (q.reverse ^ q.swaps) n = n * -1.0f;
    V3 abs_err;
    it->p = xf_point_perr(q.o2w, ph, perr, &abs_err);
    it->p_err = abs_err;
    it->time = ray.time;
    it->wo = xf_vec(q.o2w, -ray.d);
    it->n = normalize(xf_normal(q.o2w, n));
    it->surface = true;
    it->uv[0] = u;
    it->uv[1] = v;
    it->dpdu = xf_vec(q.o2w, dpdu);
    it->dpdv = xf_vec(q.o2w, dpdv);
    it->dndu = xf_normal(q.o2w, dndu);
    it->dndv = xf_normal(q.o2w, dndv);
    it->shading_n = face_forward(normalize(xf_normal(q.o2w, n)), it->n);
    it->shading_dpdu = it->dpdu;
    it->shading_dndu = it->dndu;
    it->shading_dndv = it->dndv;
}
static bool quadric_intersect(const Quadric& q, const Ray& rw, float* t_hit, Interaction* it, bool test_only) {
    V3 oe, de;
    Ray ray = xf_ray_err(q.w2o, rw, &oe, &de);
    if (q.kind == 1) {  // Disk::intersect (disk.rs:70-144)
        if (ray.d.z == 0.0f) return false;
        float tsh = (q.height - ray.o.z) / ray.d.z;
        if (tsh <= 0.0f || tsh >= ray.t_max) return false;
        V3 ph = ray.o + ray.d * tsh;
        float dist = ph.x * ph.x + ph.y * ph.y;
        if (dist > q.radius * q.radius || dist < q.inner * q.inner) return false;
        float phi = std::atan2(ph.y, ph.x);
        if (phi < 0.0f) phi += 2.0f * PI;
        if (phi > q.phi_max) return false;
        if (test_only) return true;
        float rh = std::sqrt(dist);
        float u = phi / q.phi_max, v = (q.radius - rh) / (q.radius - q.inner);  // disk.rs:106-113
        V3 dpdu(-q.phi_max * ph.y, q.phi_max * ph.x, 0.0f);
        V3 dpdv = V3(ph.x, ph.y, 0.0f) * (q.inner - q.radius) / rh;
        ph.z = q.height;
        quadric_interaction(q, ph, V3(0, 0, 0), ray, dpdu, dpdv, u, v, V3(0, 0, 0), V3(0, 0, 0), it);
        *t_hit = tsh;
        return true;
    }
    EFloat ox(ray.o.x, oe.x), oy(ray.o.y, oe.y), oz(ray.o.z, oe.z);
    EFloat dx(ray.d.x, de.x), dy(ray.d.y, de.y), dz(ray.d.z, de.z);
    EFloat a, b, c;
    if (q.kind == 0) {  // cylinder.rs:71-90
        a = dx * dx + dy * dy;
        b = ef(2.0f) * (dx * ox + dy * oy);
        c = ox * ox + oy * oy - EFloat(q.radius, 0.0f) * EFloat(q.radius, 0.0f);
    } else {  // cone.rs:67-95
        EFloat k = EFloat(q.radius, 0.0f) / EFloat(q.height, 0.0f);
        k = k * k;
        a = dx * dx + dy * dy - k * dz * dz;
        b = ef(2.0f) * (dx * ox + dy * oy - k * dz * (oz - ef(q.height)));
        c = ox * ox + oy * oy - k * (oz - ef(q.height)) * (oz - ef(q.height));
    }
    EFloat t0, t1;
    if (!quadratic(a, b, c, &t0, &t1)) return false;
    if (t0.high > ray.t_max || t1.low <= 0.0f) return false;
    EFloat tsh = t0;
    if (tsh.low <= 0.0f) {
        tsh = t1;
        if (tsh.high > ray.t_max) return false;
    }
    auto hit_point = [&](const EFloat& t) {
        V3 ph = ray.o + ray.d * t.v;
        if (q.kind == 0) {  // refine onto the cylinder
            float hr = std::sqrt(ph.x * ph.x + ph.y * ph.y);
            ph.x *= q.radius / hr;
            ph.y *= q.radius / hr;
        }
        return ph;
    };
    auto clipped = [&](V3 ph, float phi) {
        if (q.kind == 0) return ph.z < q.z_min || ph.z > q.z_max || phi > q.phi_max;
        return ph.z < 0.0f || ph.z > q.height || phi > q.phi_max;
    };
    V3 ph = hit_point(tsh);
    float phi = std::atan2(ph.y, ph.x);
    if (phi < 0.0f) phi += 2.0f * PI;
    if (clipped(ph, phi)) {
        if (tsh.v == t1.v && tsh.low == t1.low && tsh.high == t1.high) return false;
        if (t1.high > ray.t_max) return false;
        tsh = t1;
        ph = hit_point(tsh);
        phi = std::atan2(ph.y, ph.x);
        if (phi < 0.0f) phi += 2.0f * PI;
        if (clipped(ph, phi)) return false;
    }
    if (test_only) return true;
    V3 dpdu(-q.phi_max * ph.y, q.phi_max * ph.x, 0.0f), dpdv, perr, d2pduv(0, 0, 0);
    V3 d2pduu = -q.phi_max * q.phi_max * V3(ph.x, ph.y, 0.0f);
    float u = phi / q.phi_max, v;
    if (q.kind == 0) {  // cylinder.rs:149-181
        v = (ph.z - q.z_min) / (q.z_max - q.z_min);
        dpdv = V3(0.0f, 0.0f, q.z_max - q.z_min);
        perr = gamma(3.0f) * vabs(V3(ph.x, ph.y, 0.0f));
    } else {  // cone.rs:141-194
        v = ph.z / q.height;
        dpdv = V3(-ph.x / (1.0f - v), -ph.y / (1.0f - v), q.height);
        d2pduv = q.phi_max / (1.0f - v) * V3(ph.y, -ph.x, 0.0f);
        EFloat px = ox + tsh * dx, py = oy + tsh * dy, pz = oz + tsh * dz;
        perr = V3(absolute_error(px), absolute_error(py), absolute_error(pz));
    }
    V3 dndu, dndv;
    fundamental_forms(dpdu, dpdv, d2pduu, d2pduv, V3(0, 0, 0), &dndu, &dndv);
    quadric_interaction(q, ph, perr, ray, dpdu, dpdv, u, v, dndu, dndv, it);
    *t_hit = tsh.v;
    return true;
}

// ---------------------------------------------------------------- primitives + BVH
static bool prim_intersect(const Scene& s, int64_t prim, Ray& ray, Interaction* it) {
    float t;  // GeometricPrimitive::intersect (geometric.rs:27-38)
    bool ok = prim < s.ntri ? tri_intersect(s, prim, ray, &t, it, false)
              : prim < s.ntri + s.nsph ? sphere_intersect(s.sph[prim - s.ntri], ray, &t, it, false)
                                       : quadric_intersect(s.quads[prim - s.ntri - s.nsph], ray, &t, it, false);
    if (!ok) return false;
    ray.t_max = t;
    it->prim = (int)prim;
    return true;
}
static bool prim_intersect_test(const Scene& s, int64_t prim, const Ray& ray) {
    float t;
    Interaction dummy;
    if (prim < s.ntri) return tri_intersect(s, prim, ray, &t, &dummy, true);
    if (prim < s.ntri + s.nsph) return sphere_intersect(s.sph[prim - s.ntri], ray, &t, &dummy, true);
    return quadric_intersect(s.quads[prim - s.ntri - s.nsph], ray, &t, &dummy, true);
}
static Bounds3 prim_bounds(const Scene& s, int64_t prim) {
    Bounds3 b;
    if (prim < s.ntri) {  // triangle.rs:128-133
        const V3& p0 = s.pos[3 * prim];
        const V3& p1 = s.pos[3 * prim + 1];
        const V3& p2 = s.pos[3 * prim + 2];
        b.mn = {rmin(p0.x, p1.x), rmin(p0.y, p1.y), rmin(p0.z, p1.z)};
        b.mx = {rmax(p0.x, p1.x), rmax(p0.y, p1.y), rmax(p0.z, p1.z)};
        b.unite(p2);
        return b;
    }
    const Transform* o2w;
    V3 lo, hi;
    if (prim < s.ntri + s.nsph) {
        const Sphere& sp = s.sph[prim - s.ntri];  // sphere.rs:68-78
        o2w = &sp.o2w;
        lo = V3(-sp.radius, -sp.radius, sp.z_min);
        hi = V3(sp.radius, sp.radius, sp.z_max);
    } else {
        const Quadric& q = s.quads[prim - s.ntri - s.nsph];  // cylinder.rs:61-66, disk.rs:57-62, cone.rs:57-62
        o2w = &q.o2w;
        if (q.kind == 0) { lo = V3(-q.radius, -q.radius, q.z_min); hi = V3(q.radius, q.radius, q.z_max); }
        else if (q.kind == 1) { lo = V3(-q.radius, -q.radius, q.height); hi = V3(q.radius, q.radius, q.height); }
        else { lo = V3(-q.radius, -q.radius, 0.0f); hi = V3(q.radius, q.radius, q.height); }
    }
    // Transform::transform_bounds (transform.rs:75-86)
    V3 c0 = xf_point(*o2w, lo);
    b.mn = c0; b.mx = c0;
    const V3 corners[7] = {{hi.x, lo.y, lo.z}, {lo.x, hi.y, lo.z}, {lo.x, lo.y, hi.z}, {lo.x, hi.y, hi.z},
                           {hi.x, hi.y, lo.z}, {hi.x, lo.y, hi.z}, {hi.x, hi.y, hi.z}};
    for (const V3& c : corners) b.unite(xf_point(*o2w, c));
    return b;
}

struct PrimInfo {
    uint32_t index;
    Bounds3 b;
    V3 centroid;
};
// itertools 0.10 partition: two-pointer, elements mapping to true first.
template <class F>
static size_t partition_it(PrimInfo* v, size_t n, F pred) {
    size_t front = 0, back = n, split = 0;
    while (front < back) {
        PrimInfo* f = &v[front++];
        if (!pred(*f)) {
            bool swapped = false;
            while (front < back) {
                PrimInfo* b = &v[--back];
                if (pred(*b)) {
                    std::swap(*f, *b);
                    swapped = true;
                    break;
                }
            }
            if (!swapped) return split;
        }
        ++split;
    }
    return split;
}
// BVH::build (bvh.rs:91-247) as an explicit preorder work stack; `fixed` switches the bucket
// index from `16 * (offset as usize)` (F7) to `(16.0 * offset) as usize`.  Buckets start from
// BucketInfo::default() (the reference reads uninitialised memory there, bvh.rs:149-150).
static void build_bvh(Scene& s, bool fixed) {
    const int64_t n = s.nprims();
    s.nodes.clear();
    s.order.clear();
    if (n == 0) return;
    std::vector<PrimInfo> info(n);
    for (int64_t i = 0; i < n; ++i) {
        info[i].index = (uint32_t)i;
        info[i].b = prim_bounds(s, i);
        info[i].centroid = 0.5f * info[i].b.mn + 0.5f * info[i].b.mx;  // bvh.rs:443-450
    }
    struct Task { size_t begin, end; int64_t parent; };
    std::vector<Task> stack;
    stack.push_back({0, (size_t)n, -1});
    const int NB = 16;
    while (!stack.empty()) {
        Task task = stack.back();
        stack.pop_back();
        uint32_t node_index = (uint32_t)s.nodes.size();
        s.nodes.emplace_back();
        if (task.parent >= 0) s.nodes[task.parent].offset = node_index;  // second_child_offset
        PrimInfo* pi = info.data() + task.begin;
        size_t size = task.end - task.begin;
        Bounds3 bounds;
        for (size_t i = 0; i < size; ++i) bounds.unite(pi[i].b);
        auto make_leaf = [&]() {
            Scene::Node& nd = s.nodes[node_index];
            nd.b = bounds;
            nd.offset = (uint32_t)s.order.size();
            nd.count = (uint32_t)size;
            for (size_t i = 0; i < size; ++i) s.order.push_back(pi[i].index);
        };
        if (size == 1) { make_leaf(); continue; }
        Bounds3 cb;
        for (size_t i = 0; i < size; ++i) cb.unite(pi[i].centroid);
        int dim = cb.maximum_extent();
        if (cb.mx[dim] == cb.mn[dim]) { make_leaf(); continue; }
        size_t mid = size / 2;
        if (size <= 2) {
            // select_nth_unstable_by(mid, total_cmp) on two elements
            if (pi[0].centroid[dim] > pi[1].centroid[dim]) std::swap(pi[0], pi[1]);
        } else {
            auto bucket_of = [&](const PrimInfo& p) {
                float off = cb.offset(p.centroid)[dim];
                size_t b;
                if (fixed) {
                    float f = (float)NB * off;
                    b = f <= 0.0f ? 0 : (size_t)f;  // `as usize` saturates
                } else {
                    size_t o = off >= 1.0f ? 1 : 0;  // `offset as usize` is 0 or 1 on [0,1]
                    b = (size_t)NB * o;
                }
                if (b >= (size_t)NB) b = NB - 1;
                return b;
            };
            float count[NB] = {0};
            Bounds3 bb[NB];
            for (size_t i = 0; i < size; ++i) {
                size_t b = bucket_of(pi[i]);
                count[b] += 1.0f;
                bb[b].unite(pi[i].b);
            }
            float cost[NB - 1];
            float sa = bounds.surface_area();
            for (int i = 0; i < NB - 1; ++i) {
                Bounds3 b0, b1;
                float c0 = 0.0f, c1 = 0.0f;
                for (int j = 0; j <= i; ++j) { b0.unite(bb[j]); c0 += count[j]; }
                for (int j = i + 1; j < NB; ++j) { b1.unite(bb[j]); c1 += count[j]; }
                cost[i] = 1.0f + (c0 * b0.surface_area() + c1 * b1.surface_area()) / sa;
            }
            float min_cost = cost[0];
            size_t min_b = 0;
            for (int i = 1; i < NB - 1; ++i)
                if (cost[i] < min_cost) { min_cost = cost[i]; min_b = i; }
            float leaf_cost = (float)size;
            if (size > 256 || min_cost < leaf_cost) {
                mid = partition_it(pi, size, [&](const PrimInfo& p) { return bucket_of(p) <= min_b; });
            } else {
                make_leaf();
                continue;
            }
        }
        Scene::Node& nd = s.nodes[node_index];
        nd.b = bounds;  // union of both children's bounds
        nd.count = 0;
        nd.axis = (uint32_t)dim;
        stack.push_back({task.begin + mid, task.end, (int64_t)node_index});  // second child
        stack.push_back({task.begin, task.begin + mid, -1});                // first child (next)
    }
}

// BVH::intersect (bvh.rs:281-352)
static bool scene_intersect(const Scene& s, Ray& ray, Interaction* it, Counters* cnt) {
    if (s.nodes.empty()) return false;
    bool hit = false;
    V3 inv(1.0f / ray.d.x, 1.0f / ray.d.y, 1.0f / ray.d.z);
    int neg[3] = {inv.x < 0.0f, inv.y < 0.0f, inv.z < 0.0f};
    std::vector<uint32_t> todo;
    todo.reserve(64);
    uint32_t cur = 0;
    for (;;) {
        const Scene::Node& nd = s.nodes[cur];
        if (cnt) cnt->ext_visits++;
        if (nd.b.intersect_p(ray, inv, neg)) {
            if (nd.count > 0) {
                for (uint32_t i = 0; i < nd.count; ++i) {
                    if (cnt) cnt->ext_tests++;
                    if (prim_intersect(s, s.order[nd.offset + i], ray, it)) hit = true;
                }
                if (todo.empty()) break;
                cur = todo.back();
                todo.pop_back();
            } else {
                if (neg[nd.axis]) { todo.push_back(cur + 1); cur = nd.offset; }
                else { todo.push_back(nd.offset); cur = cur + 1; }
            }
        } else {
            if (todo.empty()) break;
            cur = todo.back();
            todo.pop_back();
        }
    }
    return hit;
}
// BVH::intersect_test (bvh.rs:354-423)
static bool scene_intersect_test(const Scene& s, const Ray& ray, Counters* cnt) {
    if (s.nodes.empty()) return false;
    V3 inv(1.0f / ray.d.x, 1.0f / ray.d.y, 1.0f / ray.d.z);
    int neg[3] = {inv.x < 0.0f, inv.y < 0.0f, inv.z < 0.0f};
    std::vector<uint32_t> todo;
    todo.reserve(64);
    uint32_t cur = 0;
    for (;;) {
        const Scene::Node& nd = s.nodes[cur];
        if (cnt) cnt->sh_visits++;
        if (nd.b.intersect_p(ray, inv, neg)) {
            if (nd.count > 0) {
                for (uint32_t i = 0; i < nd.count; ++i) {
                    if (cnt) cnt->sh_tests++;
                    if (prim_intersect_test(s, s.order[nd.offset + i], ray)) return true;
                }
                if (todo.empty()) break;
                cur = todo.back();
                todo.pop_back();
            } else {
                if (neg[nd.axis]) { todo.push_back(cur + 1); cur = nd.offset; }
                else { todo.push_back(nd.offset); cur = cur + 1; }
            }
        } else {
            if (todo.empty()) break;
            cur = todo.back();
            todo.pop_back();
        }
    }
    return false;
}

// ---------------------------------------------------------------- BxDFs (src/base/bxdf.rs ...)
enum : uint8_t { BSDF_REFLECTION = 1, BSDF_TRANSMISSION = 2, BSDF_DIFFUSE = 4, BSDF_GLOSSY = 8, BSDF_SPECULAR = 16,
                 BSDF_ALL = 31 };
inline float cos_theta(V3 w) { return w.z; }
inline float cos2_theta(V3 w) { return w.z * w.z; }
inline float abs_cos_theta(V3 w) { return std::fabs(w.z); }
inline float sin2_theta(V3 w) { return rmax(0.0f, 1.0f - cos2_theta(w)); }
inline float sin_theta(V3 w) { return std::sqrt(sin2_theta(w)); }
inline float tan_theta(V3 w) { return sin_theta(w) / cos_theta(w); }
inline float tan2_theta(V3 w) { return sin2_theta(w) / cos2_theta(w); }
inline float cos_phi(V3 w) { float v = sin_theta(w); return v == 0.0f ? 1.0f : rclamp(w.x / v, -1.0f, 1.0f); }
inline float sin_phi(V3 w) { float v = sin_theta(w); return v == 0.0f ? 0.0f : rclamp(w.y / v, -1.0f, 1.0f); }
inline float cos2_phi(V3 w) { return cos_phi(w) * cos_phi(w); }
inline float sin2_phi(V3 w) { return sin_phi(w) * sin_phi(w); }
inline bool same_hemisphere(V3 a, V3 b) { return a.z * b.z > 0.0f; }
inline V3 reflect(V3 wo, V3 n) { return -wo + 2.0f * dot(wo, n) * n; }  // bxdf.rs:142-144
static bool refract(V3 wi, V3 n, float eta, V3* wt) {  // bxdf.rs:146-159
    float cos_i = dot(n, wi);
    float sin2_i = rmax(0.0f, 1.0f - cos_i * cos_i);
    float sin2_t = eta * eta * sin2_i;
    if (sin2_t >= 1.0f) return false;
    float cos_t = std::sqrt(1.0f - sin2_t);
    *wt = eta * -wi + (eta * cos_i - cos_t) * n;
    return true;
}
// bxdf.rs:165-188 (F14: REF keeps a negative cos after swapping the indices; PBRT takes |cos|)
static float fresnel_dielectric(float cos_i, float eta_i, float eta_t, Mode mode) {
    cos_i = rclamp(cos_i, -1.0f, 1.0f);
    if (!(cos_i > 0.0f)) {
        std::swap(eta_i, eta_t);
        if (mode == PBRT) cos_i = std::fabs(cos_i);
    }
    float sin_i = std::sqrt(rmax(0.0f, 1.0f - cos_i * cos_i));
    float sin_t = eta_i / eta_t * sin_i;
    if (sin_t >= 1.0f) return 1.0f;
    float cos_t = std::sqrt(rmax(0.0f, 1.0f - sin_t * sin_t));
    float rpar = ((eta_t * cos_i) - (eta_i * cos_t)) / ((eta_t * cos_i) + (eta_i * cos_t));
    float rperp = ((eta_i * cos_i) - (eta_t * cos_t)) / ((eta_i * cos_i) + (eta_t * cos_t));
    return (rpar * rpar + rperp * rperp) / 2.0f;
}
static RGB fresnel_conductor(float cos_i_in, RGB eta_i, RGB eta_t, RGB k) {  // bxdf.rs:190-217
    RGB cos_i(rclamp(cos_i_in, -1.0f, 1.0f));
    RGB eta = eta_t / eta_i;
    RGB eta_k = k / eta_i;
    RGB cos_i2 = cos_i * cos_i;
    RGB sin_i2 = RGB(1.0f) - cos_i2;
    RGB eta2 = eta * eta;
    RGB eta_k2 = eta_k * eta_k;
    RGB t0 = eta2 - eta_k2 - sin_i2;
    RGB a2b2 = rgb_sqrt(t0 * t0 + eta2 * eta_k2 * 4.0f);
    RGB t1 = a2b2 + cos_i2;
    RGB a = rgb_sqrt((a2b2 + t0) * 0.5f);
    RGB t2 = cos_i * a * 2.0f;
    RGB rs = (t1 - t2) / (t1 + t2);
    RGB t3 = cos_i2 * a2b2 + sin_i2 * sin_i2;
    RGB t4 = t2 * sin_i2;
    RGB rp = rs * (t3 - t4) / (t3 + t4);
    return (rp + rs) * 0.5f;
}
// Trowbridge-Reitz (src/base/microfacet.rs)
struct TR {
    float ax, ay;
    float D(V3 wh) const {  // :116-128
        float t2 = tan2_theta(wh);
        if (std::isinf(t2)) return 0.0f;
        float cos4 = cos2_theta(wh) * cos2_theta(wh);
        float e = (cos2_phi(wh) / (ax * ax) + sin2_phi(wh) / (ay * ay)) * t2;
        return 1.0f / (PI * ax * ay * cos4 * (1.0f + e) * (1.0f + e));
    }
    float lambda(V3 w) const {  // :130-142
        float at = std::fabs(tan_theta(w));
        if (std::isinf(at)) return 0.0f;
        float alpha = std::sqrt(cos2_phi(w) * ax * ax + sin2_phi(w) * ay * ay);
        float a2t2 = (alpha * at) * (alpha * at);
        return (-1.0f + std::sqrt(1.0f + a2t2)) / 2.0f;
    }
    // F4: REF G1 = 1/(1/lambda) (microfacet.rs:17-19); PBRT G1 = 1/(1+lambda)
    float G1(V3 w, Mode mode) const { return mode == REF ? 1.0f / (1.0f / lambda(w)) : 1.0f / (1.0f + lambda(w)); }
    float G(V3 wo, V3 wi) const { return 1.0f / (1.0f + lambda(wo) + lambda(wi)); }
    float pdf(V3 wo, V3 wh, Mode mode) const { return D(wh) * G1(wo, mode) * abs_dot(wo, wh) / abs_cos_theta(wo); }
    static void sample11(float cos_t, float u1, float u2, Mode mode, float* sx_out, float* sy_out) {  // :55-97
        if (cos_t > 0.9999f) {
            float r = std::sqrt(u1 / (1.0f - u1));
            float phi = 6.28318530718f * u2;
            *sx_out = r * std::cos(phi);
            *sy_out = r * std::sin(phi);
            return;
        }
        float sin_t = std::sqrt(rmax(1.0f - cos_t * cos_t, 0.0f));
        float tan_t = sin_t / cos_t;
        float a = 1.0f / tan_t;
        float g1 = 2.0f / (1.0f + std::sqrt(1.0f + 1.0f / (a * a)));
        float A = 2.0f * u1 / g1 - 1.0f;
        float tmp = 1.0f / (A * A - 1.0f);
        if (tmp > 1e10f) tmp = 1e10f;
        float B = tan_t;
        float D = std::sqrt(rmax(B * B * tmp * tmp - (A * A - B * B) * tmp, 0.0f));
        float sx1 = B * tmp - D;
        float sx2 = B * tmp + D;
        // F5: REF always takes slope_x_1; PBRT takes slope_x_2 unless A < 0 or it is too steep
        float sx = (mode == REF) ? sx1 : ((A < 0.0f || sx2 > 1.0f / tan_t) ? sx1 : sx2);
        float S;
        if (u2 > 0.5f) { S = 1.0f; u2 = 2.0f * (u2 - 0.5f); }
        else { S = -1.0f; u2 = 2.0f * (0.5f - u2); }
        float z = (u2 * (u2 * (u2 * 0.27385f - 0.73369f) + 0.46341f)) /
                  (u2 * (u2 * (u2 * 0.093073f + 0.309420f) - 1.000000f) + 0.597999f);
        *sx_out = sx;
        *sy_out = S * z * std::sqrt(1.0f + sx * sx);
    }
    V3 sample_vis(V3 wi, float u1, float u2, Mode mode) const {  // :99-112
        V3 ws = normalize(V3(ax * wi.x, ay * wi.y, wi.z));
        float sx, sy;
        sample11(cos_theta(ws), u1, u2, mode, &sx, &sy);
        float tmp = cos_phi(ws) * sx - sin_phi(ws) * sy;
        sy = sin_phi(ws) * sx + cos_phi(ws) * sy;
        sx = tmp;
        sx = ax * sx;
        sy = ay * sy;
        return normalize(V3(-sx, -sy, 1.0f));
    }
    V3 sample_wh(V3 wo, float u0, float u1, Mode mode) const {  // :144-153
        bool flip = wo.z < 0.0f;
        V3 w = flip ? -wo : wo;
        V3 wh = sample_vis(w, u0, u1, mode);
        return flip ? -wh : wh;
    }
};
static float roughness_to_alpha(float r) {  // microfacet.rs:45-53
    r = rmax(r, 1e-3f);
    float x = std::log(r);
    return 1.62142f + 0.819955f * x + 0.1734f * x * x + 0.0171201f * x * x * x + 0.000640711f * x * x * x * x;
}

enum BxKind { LAMBERT, MF_REFL, FRESNEL_SPEC, OREN_NAYAR, SPEC_REFL, SPEC_TRANS };
struct Bxdf {
    BxKind kind;
    uint8_t type;
    RGB r, t;
    TR dist{1, 1};
    bool conductor = false;  // fresnel kind for MF_REFL
    RGB c_eta_i, c_eta_t, c_k;
    float d_eta_i = 1, d_eta_t = 1;
    float eta_a = 1, eta_b = 1;
    float on_a = 1, on_b = 0;  // OrenNayer A, B
    bool matches(uint8_t f) const { return (type & f) == type; }
};
struct BxSample {
    V3 wi;
    RGB f;
    float pdf = 0;
    int sampled_type = -1;
};
static RGB bx_f(const Bxdf& b, V3 wo, V3 wi, Mode mode) {
    switch (b.kind) {
        case LAMBERT: return b.r * (1.0f / PI);  // lambertian.rs:42-45
        case OREN_NAYAR: {                       // oren_nayer.rs:34-60
            float sin_i = sin_theta(wi), sin_o = sin_theta(wo);
            float max_cos = 0.0f;
            if (sin_i > 1e-4f && sin_o > 1e-4f) {
                float d_cos = cos_phi(wi) * cos_phi(wo) + sin_phi(wi) * sin_phi(wo);
                max_cos = rmax(0.0f, d_cos);
            }
            float sin_alpha, tan_beta;
            if (abs_cos_theta(wi) > abs_cos_theta(wo)) {
                sin_alpha = sin_o;
                tan_beta = sin_i / abs_cos_theta(wi);
            } else {
                sin_alpha = sin_i;
                tan_beta = sin_o / abs_cos_theta(wo);
            }
            return b.r * (1.0f / PI) * (b.on_a + b.on_b * max_cos * sin_alpha * tan_beta);
        }
        case MF_REFL: {                          // bxdfs/microfacet.rs:69-94
            float co = abs_cos_theta(wo), ci = abs_cos_theta(wi);
            V3 wh = wi + wo;
            if (ci == 0.0f || co == 0.0f) return RGB();
            if (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) return RGB();
            wh = normalize(wh);
            float c = dot(wi, face_forward(wh, V3(0, 0, 1)));
            RGB F = b.conductor ? fresnel_conductor(std::fabs(c), b.c_eta_i, b.c_eta_t, b.c_k)
                                : RGB(fresnel_dielectric(c, b.d_eta_i, b.d_eta_t, mode));
            return b.r * b.dist.D(wh) * b.dist.G(wo, wi) * F / (4.0f * ci * co);
        }
        default: return RGB();
    }
}
static float bx_pdf(const Bxdf& b, V3 wo, V3 wi, Mode mode) {
    switch (b.kind) {
        case LAMBERT:
        case OREN_NAYAR: return same_hemisphere(wo, wi) ? abs_cos_theta(wi) * (1.0f / PI) : 0.0f;  // bxdf.rs:72-78
        case MF_REFL: {  // bxdfs/microfacet.rs:142-147
            if (!same_hemisphere(wo, wi)) return 0.0f;
            V3 wh = normalize(wo + wi);
            return b.dist.pdf(wo, wh, mode) / (4.0f * dot(wo, wh));
        }
        default: return 0.0f;
    }
}
static V3 concentric_sample_disk(float u0, float u1, float* dy) {  // sampling.rs:181-198
    float ox = 2.0f * u0 - 1.0f, oy = 2.0f * u1 - 1.0f;
    if (ox == 0.0f && oy == 0.0f) { *dy = 0.0f; return V3(); }
    float theta, r;
    if (std::fabs(ox) > std::fabs(oy)) { theta = (PI / 4.0f) * (oy / ox); r = ox; }
    else { theta = PI_OVER_TWO - (PI / 4.0f) * (ox / oy); r = oy; }
    *dy = r * std::sin(theta);
    return V3(r * std::cos(theta), 0, 0);
}
static V3 cosine_sample_hemisphere(float u0, float u1) {  // sampling.rs:238-242
    float dy;
    float dx = concentric_sample_disk(u0, u1, &dy).x;
    float z = std::sqrt(rmax(0.0f, 1.0f - dx * dx - dy * dy));
    return V3(dx, dy, z);
}
static BxSample bx_sample(const Bxdf& b, V3 wo, float u0, float u1, Mode mode) {
    BxSample s;
    switch (b.kind) {
        case SPEC_REFL: {  // specular.rs:57-66
            V3 wi(-wo.x, -wo.y, wo.z);
            s.wi = wi;
            s.f = RGB(fresnel_dielectric(cos_theta(wi), b.eta_a, b.eta_b, mode)) * b.r / abs_cos_theta(wi);
            s.pdf = 1.0f;
            return s;
        }
        case SPEC_TRANS: {  // specular.rs:82-113
            bool entering = cos_theta(wo) > 0.0f;
            float ei = entering ? b.eta_a : b.eta_b, et = entering ? b.eta_b : b.eta_a;
            V3 wi;
            if (!refract(wo, face_forward(V3(0, 0, 1), wo), ei / et, &wi)) return s;
            RGB f = b.t * (RGB(1.0f) - RGB(fresnel_dielectric(cos_theta(wi), b.eta_a, b.eta_b, mode)));
            f = f * ((ei * ei) / (et * et));
            s.wi = wi;
            s.f = f / abs_cos_theta(wi);
            s.pdf = 1.0f;
            return s;
        }
        case OREN_NAYAR:
        case LAMBERT: {  // default BxDF::sample (bxdf.rs:33-45)
            V3 wi = cosine_sample_hemisphere(u0, u1);
            if (wo.z < 0.0f) wi.z *= -1.0f;
            s.wi = wi;
            s.f = bx_f(b, wo, wi, mode);
            s.pdf = bx_pdf(b, wo, wi, mode);
            return s;
        }
        case MF_REFL: {  // bxdfs/microfacet.rs:96-140
            if (wo.z == 0.0f) return s;
            V3 wh = b.dist.sample_wh(wo, u0, u1, mode);
            if (dot(wo, wh) < 0.0f) return s;
            V3 wi = reflect(wo, wh);
            if (!same_hemisphere(wo, wi)) return s;
            s.wi = wi;
            s.f = bx_f(b, wo, wi, mode);
            s.pdf = b.dist.pdf(wo, wh, mode) / (4.0f * dot(wo, wh));
            return s;
        }
        case FRESNEL_SPEC: {  // bxdfs/fresnel.rs:76-122
            float F = fresnel_dielectric(cos_theta(wo), b.eta_a, b.eta_b, mode);
            if (u0 < F) {
                V3 wi(-wo.x, -wo.y, wo.z);
                s.wi = wi;
                s.pdf = F;
                s.f = RGB(F) * b.r / abs_cos_theta(wi);
                s.sampled_type = BSDF_SPECULAR | BSDF_REFLECTION;
                return s;
            }
            bool entering = cos_theta(wo) > 0.0f;
            float ei = entering ? b.eta_a : b.eta_b, et = entering ? b.eta_b : b.eta_a;
            V3 wi;
            if (!refract(wo, face_forward(V3(0, 0, 1), wo), ei / et, &wi)) return s;
            RGB ft = b.t * (1.0f - F);
            ft = ft * ((ei * ei) / (et * et));
            s.wi = wi;
            s.f = ft / abs_cos_theta(wi);
            s.pdf = 1.0f - F;
            s.sampled_type = BSDF_SPECULAR | BSDF_TRANSMISSION;
            return s;
        }
    }
    return s;
}

struct BSDF {  // src/base/bsdf.rs
    float eta = 1.0f;
    V3 ns, ng, ss, ts;
    Bxdf bx[2];
    int n = 0;
    int num_components(uint8_t f) const {
        int k = 0;
        for (int i = 0; i < n; ++i) k += bx[i].matches(f);
        return k;
    }
    V3 to_local(V3 v) const { return V3(dot(v, ss), dot(v, ts), dot(v, ns)); }
    V3 to_world(V3 v) const {
        return V3(ss.x * v.x + ts.x * v.y + ns.x * v.z, ss.y * v.x + ts.y * v.y + ns.y * v.z,
                  ss.z * v.x + ts.z * v.y + ns.z * v.z);
    }
    RGB f(V3 wo_w, V3 wi_w, uint8_t flags, Mode mode) const {  // bsdf.rs:84-105
        V3 wo = to_local(wo_w), wi = to_local(wi_w);
        if (wo.z == 0.0f) return RGB();
        bool refl = dot(wi_w, ng) * dot(wo_w, ng) > 0.0f;
        RGB r;
        for (int i = 0; i < n; ++i)
            if (bx[i].matches(flags) && ((refl && (bx[i].type & BSDF_REFLECTION)) ||
                                         (!refl && (bx[i].type & BSDF_TRANSMISSION))))
                r = r + bx_f(bx[i], wo, wi, mode);
        return r;
    }
    float pdf(V3 wo_w, V3 wi_w, uint8_t flags, Mode mode) const {  // bsdf.rs:234-259
        if (n == 0) return 0.0f;
        V3 wo = to_local(wo_w), wi = to_local(wi_w);
        if (wo.z == 0.0f) return 0.0f;
        float ret = 0.0f, comps = 0.0f;
        for (int i = 0; i < n; ++i)
            if (bx[i].matches(flags)) { comps += 1.0f; ret += bx_pdf(bx[i], wo, wi, mode); }
        return comps > 0.0f ? ret / comps : 0.0f;
    }
    BxSample sample(V3 wo_w, float u0, float u1, uint8_t type, Mode mode) const {  // bsdf.rs:140-232
        BxSample zero;
        zero.sampled_type = 0;
        int matches = num_components(type);
        if (matches == 0) return zero;
        uint32_t comp = std::min((uint32_t)std::floor(u0 * (float)matches), (uint32_t)matches - 1);
        // F8: REF decrements the counter for every BxDF (u32), PBRT only for matching ones
        uint32_t count = comp;
        int pick = -1;
        for (int i = 0; i < n; ++i) {
            if (bx[i].matches(type) && count == 0) { pick = i; break; }
            if (mode == REF || bx[i].matches(type)) count -= 1;
        }
        if (pick < 0) return zero;  // the reference panics here (bsdf.rs:162)
        const Bxdf& b = bx[pick];
        float ur0 = rmin(u0 * (float)matches - (float)comp, ONE_MINUS_EPSILON);
        V3 wo = to_local(wo_w);
        if (wo.z == 0.0f) return zero;
        BxSample s = bx_sample(b, wo, ur0, u1, mode);
        int stype = s.sampled_type >= 0 ? s.sampled_type : b.type;
        if (s.pdf == 0.0f) return zero;
        V3 wi_w = to_world(s.wi);
        if (!(b.type & BSDF_SPECULAR) && matches > 1)
            for (int i = 0; i < n; ++i)
                if (i != pick && bx[i].matches(type)) s.pdf += bx_pdf(bx[i], wo, s.wi, mode);
        if (matches > 1) s.pdf /= (float)matches;
        if (!(b.type & BSDF_SPECULAR)) {
            bool refl = dot(wi_w, ng) * dot(wo_w, ng) > 0.0f;
            s.f = RGB();
            for (int i = 0; i < n; ++i)
                if (bx[i].matches(type) && ((refl && (bx[i].type & BSDF_REFLECTION)) ||
                                            (!refl && (bx[i].type & BSDF_TRANSMISSION))))
                    s.f = s.f + bx_f(bx[i], wo, s.wi, mode);
        }
        s.wi = wi_w;
        s.sampled_type = stype;
        return s;
    }
};
// ---------------------------------------------------------------- ray differentials + textures
struct RayDifferential {  // ray.rs:7-13
    bool has = false;
    V3 rxo, ryo, rxd, ryd;
};
// solve_linear_system_2x2 (src/base/math.rs:52-68)
static bool solve_2x2(const float a[2][2], const float b[2], float* x0, float* x1) {
    float det = a[0][0] * a[1][1] - a[0][1] * a[1][0];
    if (std::fabs(det) < 1e-10f) return false;
    *x0 = (a[1][1] * b[0] - a[0][1] * b[1]) / det;
    *x1 = (a[0][0] * b[1] - a[1][0] * b[0]) / det;
    if (std::isnan(*x0) || std::isnan(*x1)) return false;
    return true;
}
// Interaction::compute_differentials (interaction.rs:184-250)
static void compute_differentials(Interaction* it, const RayDifferential& rd) {
    it->dudx = it->dvdx = it->dudy = it->dvdy = 0.0f;
    it->dpdx = it->dpdy = V3(0, 0, 0);
    if (!rd.has) return;
    float d = dot(it->n, it->p);
    float tx = -(dot(it->n, rd.rxo) - d) / dot(it->n, rd.rxd);
    if (std::isinf(tx) || std::isnan(tx)) return;
    V3 px = rd.rxo + tx * rd.rxd;
    float ty = -(dot(it->n, rd.ryo) - d) / dot(it->n, rd.ryd);
    if (std::isinf(ty) || std::isnan(ty)) return;
    V3 py = rd.ryo + ty * rd.ryd;
    it->dpdx = px - it->p;
    it->dpdy = py - it->p;
    const V3& n = it->n;
    int dim[2];
    if (std::fabs(n.x) > std::fabs(n.y) && std::fabs(n.x) > std::fabs(n.z)) { dim[0] = 1; dim[1] = 2; }
    else if (std::fabs(n.y) > std::fabs(n.z)) { dim[0] = 0; dim[1] = 2; }
    else { dim[0] = 0; dim[1] = 1; }
    float a[2][2] = {{it->dpdu[dim[0]], it->dpdv[dim[0]]}, {it->dpdu[dim[1]], it->dpdv[dim[1]]}};
    float bx[2] = {px[dim[0]] - it->p[dim[0]], px[dim[1]] - it->p[dim[1]]};
    float by[2] = {py[dim[0]] - it->p[dim[0]], py[dim[1]] - it->p[dim[1]]};
    if (!solve_2x2(a, bx, &it->dudx, &it->dvdx)) it->dudx = it->dvdx = 0.0f;
    if (!solve_2x2(a, by, &it->dudy, &it->dvdy)) it->dudy = it->dvdy = 0.0f;
}

// `as i32` (saturating, NaN -> 0)
static int32_t to_i32(float f) {
    if (std::isnan(f)) return 0;
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f <= -2147483648.0f) return INT32_MIN;
    return (int32_t)f;
}
static int32_t modulo_i32(int32_t a, int32_t b) {  // math.rs:43-50
    int32_t r = a - (a / b) * b;
    return r < 0 ? r + b : r;
}
// Image::get_channel with remap_pixel (image.rs:130-159)
static float image_channel(const Image& im, int32_t x, int32_t y, int c, uint32_t wrap) {
    int32_t p[2] = {x, y};
    const int32_t res[2] = {im.w, im.h};
    for (int k = 0; k < 2; ++k) {
        if (p[k] >= 0 && p[k] < res[k]) continue;
        if (wrap == BG_WRAP_REPEAT) p[k] = modulo_i32(p[k], res[k]);
        else if (wrap == BG_WRAP_CLAMP) p[k] = p[k] < 0 ? 0 : (p[k] > res[k] - 1 ? res[k] - 1 : p[k]);
        else return 0.0f;
    }
    return im.px[3 * ((size_t)p[1] * im.w + p[0]) + c];
}
static RGB mip_texel(const Texture& t, size_t level, int32_t x, int32_t y) {  // mipmap.rs:175-182
    const Image& im = t.pyramid[level];
    return RGB(image_channel(im, x, y, 0, t.wrap), image_channel(im, x, y, 1, t.wrap),
               image_channel(im, x, y, 2, t.wrap));
}
static RGB mip_triangle(const Texture& t, size_t level, float st0, float st1) {  // mipmap.rs:156-173
    level = std::min(level, t.pyramid.size() - 1);
    const Image& im = t.pyramid[level];
    float sx = st0 * (float)im.w - 0.5f, sy = st1 * (float)im.h - 0.5f;
    float ds = sx - std::floor(sx), dt = sy - std::floor(sy);
    int32_t s0 = to_i32(std::floor(sx)), t0 = to_i32(std::floor(sy));
    int32_t s1 = (int32_t)((uint32_t)s0 + 1u), t1 = (int32_t)((uint32_t)t0 + 1u);
    return (1.0f - ds) * (1.0f - dt) * mip_texel(t, level, s0, t0) + (1.0f - ds) * dt * mip_texel(t, level, s0, t1) +
           ds * (1.0f - dt) * mip_texel(t, level, s1, t0) + ds * dt * mip_texel(t, level, s1, t1);
}
// MIPMap::filter / trilinear_filter (mipmap.rs:103-128)
static RGB mip_trilinear(const Texture& t, float st0, float st1, float width) {
    const float top = (float)(t.pyramid.size() - 1);
    float level = top + std::log2(rmax(width, 1e-8f));
    if (level < 0.0f) return mip_triangle(t, 0, st0, st1);
    if (level >= top) return mip_texel(t, t.pyramid.size() - 1, 0, 0);
    size_t il = (size_t)std::floor(level);
    float f = level - std::floor(level);
    return (1.0f - f) * mip_triangle(t, il, st0, st1) + f * mip_triangle(t, il + 1, st0, st1);
}
static RGB mip_filter(const Texture& t, float st0, float st1, const float d0[2], const float d1[2]) {
    float width = rmax(rmax(std::fabs(d0[0]), std::fabs(d0[1])), rmax(std::fabs(d1[0]), std::fabs(d1[1])));
    return mip_trilinear(t, st0, st1, width);
}
// SphericalMapping2D::sphere / CylindricalMapping2D::cylinder (texture.rs:48-62)
static void map_sphere(const Texture& t, V3 p, Mode mode, float st[2]) {
    V3 v = normalize(xf_point(t.w2t, p) - V3(0, 0, 0));
    float theta = std::acos(rclamp(v.z, -1.0f, 1.0f));
    float phi = std::atan2(v.y, v.x);
    if (phi < 0.0f) phi = phi + 2.0f * PI;
    st[0] = theta * (1.0f / PI);
    st[1] = phi * (mode == REF ? (1.0f / PI) : (1.0f / (2.0f * PI)));  // REF: phi / pi as written
}
static void map_cylinder(const Texture& t, V3 p, float st[2]) {
    V3 v = normalize(xf_point(t.w2t, p) - V3(0, 0, 0));
    st[0] = (PI + std::atan2(v.y, v.x)) * (1.0f / (2.0f * PI));
    st[1] = v.z;
}
// TextureMapping2D::map (texture.rs:64-144)
static void tex_map(const Texture& t, const Interaction& it, Mode mode, float st[2], float dx[2], float dy[2]) {
    if (t.mapping == BG_MAPPING_UV) {
        dx[0] = t.su * it.dudx;
        dx[1] = t.sv * it.dvdx;
        dy[0] = t.su * it.dudy;
        dy[1] = t.sv * it.dvdy;
        st[0] = t.su * it.uv[0] + t.du;
        st[1] = t.sv * it.uv[1] + t.dv;
        return;
    }
    if (t.mapping == BG_MAPPING_PLANAR) {
        dx[0] = dot(it.dpdx, t.vs);
        dx[1] = dot(it.dpdx, t.vt);
        dy[0] = dot(it.dpdy, t.vs);
        dy[1] = dot(it.dpdy, t.vt);
        st[0] = t.ds + dot(it.p, t.vs);
        st[1] = t.dt + dot(it.p, t.vt);
        return;
    }
    const float DELTA = 0.1f;
    auto at = [&](V3 p, float o[2]) {
        if (t.mapping == BG_MAPPING_SPHERICAL) map_sphere(t, p, mode, o);
        else map_cylinder(t, p, o);
    };
    float sx[2], sy[2];
    at(it.p, st);
    at(it.p + DELTA * it.dpdx, sx);
    at(it.p + DELTA * it.dpdy, sy);
    for (int k = 0; k < 2; ++k) {
        dx[k] = (sx[k] - st[k]) / DELTA;
        dy[k] = (sy[k] - st[k]) / DELTA;
    }
    for (float* d : {dx, dy}) {  // mapping discontinuity of the second coordinate
        if (d[1] > 0.5f) d[1] = 1.0f - d[1];
        else if (d[1] < -0.5f) d[1] = -(d[1] + 1.0f);
    }
}
// Texture<RGBSpectrum>::evaluate (image.rs:35-42, uv.rs:8-15)
static RGB tex_eval(const Scene& s, uint32_t id, const Interaction& it, Mode mode) {
    const Texture& t = s.tex[id];
    float st[2], dx[2], dy[2];
    tex_map(t, it, mode, st, dx, dy);
    if (t.kind == BG_TEXTURE_UV) return RGB(st[0] - std::floor(st[0]), st[1] - std::floor(st[1]), 0.0f);
    return mip_filter(t, st[0], st[1], dx, dy);
}
// Image::generate_pyramid (image.rs:55-114)
static std::vector<Image> generate_pyramid(Image img) {
    size_t levels = 1;
    for (int m = std::max(img.w, img.h); m > 1; m >>= 1) ++levels;
    std::vector<Image> pyr;
    pyr.push_back(std::move(img));
    for (size_t i = 1; i < levels; ++i) {
        const Image& last = pyr[i - 1];
        Image next;
        next.w = std::max(last.w / 2, 1);
        next.h = std::max(last.h / 2, 1);
        next.px.assign((size_t)next.w * next.h * 3, 0.0f);
        size_t deltas[4] = {0, 3, 3 * (size_t)last.w, 3 * ((size_t)last.w + 1)};
        if (last.w == 1) { deltas[1] = 0; deltas[3] -= 3; }
        if (last.h == 1) { deltas[2] = 0; deltas[3] -= 3 * (size_t)last.w; }
        for (int y = 0; y < next.h; ++y) {
            size_t src = 3 * ((size_t)(2 * y) * last.w), dst = 3 * ((size_t)y * next.w);
            for (int x = 0; x < next.w; ++x) {
                for (int c = 0; c < 3; ++c) {
                    next.px[dst] = (last.px[src] + last.px[src + deltas[1]] + last.px[src + deltas[2]] +
                                    last.px[src + deltas[3]]) * 0.25f;
                    ++src;
                    ++dst;
                }
                src += 3;
            }
        }
        pyr.push_back(std::move(next));
    }
    return pyr;
}

// Material::compute_scattering_functions (materials/matte.rs:19-41, plastic.rs:65-95 and the
// composed conductor / dielectric)
// `it` carries the differentials (compute_differentials) that textures read; multi_lobe =
// allow_multiple_lobes (false for the Whitted and direct-lighting integrators).
static BSDF make_bsdf(const Scene& s, const Interaction& it, Mode mode = PBRT, bool multi_lobe = true) {
    const bg_material& m = s.mats[it.prim < s.ntri ? s.tri_mat[it.prim]
                                  : it.prim < s.ntri + s.nsph ? s.sph[it.prim - s.ntri].mat
                                                              : s.quads[it.prim - s.ntri - s.nsph].mat];
    BSDF b;
    b.ns = it.shading_n;
    b.ng = it.n;
    b.ss = normalize(it.shading_dpdu);
    b.ts = cross(b.ns, b.ss);
    auto clamp0 = [](RGB c) {  // RGBSpectrum::clamp(0, inf)
        return RGB(rclamp(c.c[0], 0.0f, INFINITY), rclamp(c.c[1], 0.0f, INFINITY), rclamp(c.c[2], 0.0f, INFINITY));
    };
    auto texture = [&](uint32_t id, const float* constant) {  // ConstantTexture or textures[id - 1]
        return id ? tex_eval(s, id - 1, it, mode) : RGB(constant[0], constant[1], constant[2]);
    };
    if (m.type == BG_MAT_MATTE || m.type == BG_MAT_PLASTIC) {
        RGB kd = clamp0(texture(m.kd_texture, m.kd));
        if (!kd.is_black()) {
            Bxdf l;
            l.kind = LAMBERT;
            l.type = BSDF_REFLECTION | BSDF_DIFFUSE;
            l.r = kd;
            float sigma = m.type == BG_MAT_MATTE ? rclamp(m.sigma, 0.0f, 90.0f) : 0.0f;
            if (sigma != 0.0f) {  // OrenNayer::new (oren_nayer.rs:20-30)
                l.kind = OREN_NAYAR;
                float rad = sigma * (PI / 180.0f);
                float s2 = rad * rad;
                l.on_a = 1.0f - (s2 / (2.0f * (s2 + 0.33f)));
                l.on_b = 0.45f * s2 / (s2 + 0.09f);
            }
            b.bx[b.n++] = l;
        }
        if (m.type == BG_MAT_PLASTIC) {
            RGB ks = clamp0(texture(m.ks_texture, m.ks));
            if (!ks.is_black()) {
                float rough = m.roughness;
                if (m.remap_roughness) rough = roughness_to_alpha(rough);
                Bxdf g;
                g.kind = MF_REFL;
                g.type = BSDF_REFLECTION | BSDF_GLOSSY;
                g.r = ks;
                g.dist = TR{rmax(rough, 0.001f), rmax(rough, 0.001f)};
                g.conductor = false;
                g.d_eta_i = 1.5f;
                g.d_eta_t = 1.0f;
                b.bx[b.n++] = g;
            }
        }
    } else if (m.type == BG_MAT_CONDUCTOR) {
        Bxdf g;
        g.kind = MF_REFL;
        g.type = BSDF_REFLECTION | BSDF_GLOSSY;
        g.r = RGB(1.0f);
        g.dist = TR{rmax(m.roughness, 0.001f), rmax(m.roughness, 0.001f)};
        g.conductor = true;
        g.c_eta_i = RGB(1.0f);
        g.c_eta_t = RGB(m.eta[0], m.eta[1], m.eta[2]);
        g.c_k = RGB(m.k[0], m.k[1], m.k[2]);
        b.bx[b.n++] = g;
    } else if (mode == REF || multi_lobe) {  // dielectric
        b.eta = m.ior;
        Bxdf d;
        d.kind = FRESNEL_SPEC;
        d.type = BSDF_REFLECTION | BSDF_TRANSMISSION | BSDF_SPECULAR;
        d.r = RGB(1.0f);
        d.t = RGB(1.0f);
        d.eta_a = 1.0f;
        d.eta_b = m.ior;
        b.bx[b.n++] = d;
    } else {  // dielectric without multiple lobes: SpecularReflection + SpecularTransmission
        b.eta = m.ior;
        Bxdf r;
        r.kind = SPEC_REFL;
        r.type = BSDF_REFLECTION | BSDF_SPECULAR;
        r.r = RGB(1.0f);
        r.eta_a = 1.0f;
        r.eta_b = m.ior;
        b.bx[b.n++] = r;
        Bxdf t;
        t.kind = SPEC_TRANS;
        t.type = BSDF_TRANSMISSION | BSDF_SPECULAR;
        t.t = RGB(1.0f);
        t.eta_a = 1.0f;
        t.eta_b = m.ior;
        b.bx[b.n++] = t;
    }
    return b;
}

// ---------------------------------------------------------------- lights (src/lights/diffuse.rs)
static RGB emission(const bg_area_light& l, V3 n, V3 dir) {  // diffuse.rs:163-169
    if (l.two_sided || dot(n, dir) > 0.0f) return RGB(l.intensity[0], l.intensity[1], l.intensity[2]);
    return RGB();
}
static RGB emitted_radiance(const Scene& s, const Interaction& it, V3 w) {  // interaction.rs:257-266
    if (it.prim < 0) return RGB();
    int32_t e = s.prim_emission[it.prim];
    if (e < 0) return RGB();
    return emission(s.emis[e], it.n, w);
}
struct LightSample {
    RGB radiance;
    V3 wi;
    float pdf = 0.0f;
    Interaction p0, p1;
    bool vis = false;
};
// ---- shapes as area lights: Shape::sample (sphere.rs:328-355, disk.rs:184-214,
// cylinder.rs:289-321) and area (sphere.rs:375-377, disk.rs:216-218, cylinder.rs:323-325).
// F21 (REF): sphere and cylinder sample normals are not normalised.  F22 (REF): the disk draws
// from the whole disk of the outer radius; PBRT draws the annulus sector uniformly.
static float sphere_area(const Sphere& sp) { return sp.phi_max * sp.radius * (sp.z_max - sp.z_min); }
static float quadric_area(const Quadric& q) {
    if (q.kind == 1) return q.phi_max * 0.5f * (q.radius * q.radius - q.inner * q.inner);
    return (q.z_max - q.z_min) * q.radius * q.phi_max;
}
static Interaction sphere_sample(const Sphere& sp, float u0, float u1, Mode mode, float* pdf) {
    float z = 1.0f - 2.0f * u0;  // uniform_sample_sphere (sampling.rs:211-216)
    float rr = std::sqrt(rmax(1.0f - z * z, 0.0f));
    float phi = 2.0f * PI * u1;
    V3 obj(0.0f + sp.radius * (rr * std::cos(phi)), 0.0f + sp.radius * (rr * std::sin(phi)), 0.0f + sp.radius * z);
    Interaction r;
    r.n = xf_normal(sp.o2w, obj);
    if (mode == PBRT) r.n = normalize(r.n);
    float k = sp.radius / length(obj);
    obj = V3(obj.x * k, obj.y * k, obj.z * k);
    V3 oerr = gamma(5.0f) * vabs(obj);
    r.p = xf_point_perr(sp.o2w, obj, oerr, &r.p_err);
    *pdf = 1.0f / sphere_area(sp);
    return r;
}
static Interaction quadric_sample(const Quadric& q, float u0, float u1, Mode mode, float* pdf) {
    Interaction r;
    V3 obj, oerr(0.0f, 0.0f, 0.0f);
    if (q.kind == 1) {  // disk
        if (mode == REF) {
            float dy;
            float dx = concentric_sample_disk(u0, u1, &dy).x;
            obj = V3(dx * q.radius, dy * q.radius, q.height);
        } else {
            float rad = std::sqrt((1.0f - u0) * (q.inner * q.inner) + u0 * (q.radius * q.radius));
            float ph = u1 * q.phi_max;
            obj = V3(rad * std::cos(ph), rad * std::sin(ph), q.height);
        }
        r.n = normalize(xf_normal(q.o2w, V3(0.0f, 0.0f, 1.0f)));
    } else {  // cylinder
        float z = (1.0f - u0) * q.z_min + u0 * q.z_max;
        float phi = u1 * q.phi_max;
        obj = V3(q.radius * std::cos(phi), q.radius * std::sin(phi), z);
        r.n = xf_normal(q.o2w, V3(obj.x, obj.y, 0.0f));
        if (mode == PBRT) r.n = normalize(r.n);
        float hr = std::sqrt(obj.x * obj.x + obj.y * obj.y);
        obj.x *= q.radius / hr;
        obj.y *= q.radius / hr;
        oerr = gamma(3.0f) * vabs(V3(obj.x, obj.y, 0.0f));
    }
    if (q.reverse) r.n = r.n * -1.0f;
    r.p = xf_point_perr(q.o2w, obj, oerr, &r.p_err);
    *pdf = 1.0f / quadric_area(q);
    return r;
}

// ---- InfiniteAreaLight (src/lights/infinite.rs) over Distribution2D (src/base/sampling.rs)
// find_interval (math.rs:70-87): the last index i < size - 1 with cdf[i] <= u
static size_t cdf_interval(const float* cdf, size_t size, float u) {
    size_t lo = 0, len = size;
    while (len > 0) {
        size_t half = len / 2;
        if (cdf[lo + half] <= u) {
            lo = lo + half + 1;
            len = len - half - 1;
        } else {
            len = half;
        }
    }
    size_t r = lo == 0 ? 0 : lo - 1;  // cdf[0] = 0 <= u, so lo >= 1 for u >= 0
    return r > size - 2 ? size - 2 : r;
}
// Distribution1D::sample_continuous (sampling.rs:53-76); count = Distribution1D::count
static float d1_sample(const float* cdf, const float* func, float func_int, size_t n, size_t count, float u,
                       float* pdf, size_t* off) {
    size_t o = cdf_interval(cdf, n + 1, u);
    if (off) *off = o;
    float du = u - cdf[o];
    if (cdf[o + 1] - cdf[o] > 0.0f) du /= cdf[o + 1] - cdf[o];
    *pdf = func_int > 0.0f ? func[o] / func_int : 0.0f;
    return ((float)o + du) / (float)count;
}
// Distribution2D::sample_continuous (sampling.rs:99-111).  F18 (REF): conditional v holds the
// function's whole tail (func[v * nu..], sampling.rs:84), so its count is (nv - v) * nu.
static void d2_sample(const InfiniteLight& L, float u0, float u1, Mode mode, float uv[2], float* pdf) {
    float p1, p0;
    size_t v = 0;
    uv[1] = d1_sample(L.marg_cdf.data(), L.cond_int.data(), L.marg_int, L.nv, L.nv, u1, &p1, &v);
    size_t count = mode == REF ? (size_t)(L.nv - v) * L.nu : L.nu;
    uv[0] = d1_sample(&L.cond_cdf[v * (L.nu + 1)], &L.func[v * L.nu], L.cond_int[v], L.nu, count, u0, &p0, nullptr);
    *pdf = p0 * p1;
}
// Distribution2D::pdf (sampling.rs:113-117).  F19 (REF): `p[0] as usize * count` truncates p
// before scaling: the cell is 0 unless a coordinate is >= 1, and the column bound is conditional
// 0's count (nv * nu under F18).  An index past row v's tail (a panic in the reference) reads the
// function's last entry.
static float d2_pdf(const InfiniteLight& L, float p0, float p1, Mode mode) {
    size_t idx;
    if (mode == REF) {
        auto trunc = [](float x) -> size_t { return x >= 1.0f ? (size_t)x : 0; };
        size_t cu = (size_t)L.nv * L.nu, cv = L.nv;
        size_t u = std::min(trunc(p0) * cu, cu - 1), v = std::min(trunc(p1) * cv, cv - 1);
        idx = std::min(v * L.nu + u, (size_t)L.nv * L.nu - 1);
    } else {
        int64_t u = (int64_t)(p0 * (float)L.nu), v = (int64_t)(p1 * (float)L.nv);
        u = std::max<int64_t>(0, std::min<int64_t>(u, L.nu - 1));
        v = std::max<int64_t>(0, std::min<int64_t>(v, L.nv - 1));
        idx = (size_t)v * L.nu + (size_t)u;
    }
    return L.func[idx] / L.marg_int;
}
static float sph_theta(V3 v) { return std::acos(rclamp(v.z, -1.0f, 1.0f)); }  // geometry.rs:6-8
static float sph_phi(V3 v) {                                                     // geometry.rs:10-17
    float p = std::atan2(v.y, v.x);
    return p < 0.0f ? p + 2.0f * PI : p;
}
// InfiniteAreaLight::radiance (infinite.rs:88-96)
static RGB inf_radiance(const Scene& s, V3 dir) {
    V3 w = normalize(xf_vec(s.inf.w2l, dir));
    return mip_trilinear(s.inf.map, sph_phi(w) * (1.0f / (2.0f * PI)), sph_theta(w) * (1.0f / PI), 0.0f);
}
// Light::radiance summed over the scene's lights for an escaping ray: only the infinite light's
// is non-zero (area lights return zero, light.rs:31-33).
static RGB escaped_radiance(const Scene& s, V3 dir) { return s.has_inf ? inf_radiance(s, dir) : RGB(); }

static LightSample light_sample_point(const Scene& s, int64_t prim, const Interaction& it, float u0, float u1,
                                      Mode mode) {  // diffuse.rs:54-87 + shape.rs:17-34
    LightSample ls;
    if (prim == LIGHT_INF) {  // InfiniteAreaLight::sample_point (infinite.rs:98-153)
        const InfiniteLight& L = s.inf;
        float uv[2], map_pdf;
        d2_sample(L, u0, u1, mode, uv, &map_pdf);
        if (map_pdf == 0.0f) return ls;
        float theta = uv[1] * PI, phi = uv[0] * 2.0f * PI;
        float st = std::sin(theta), ct = std::cos(theta), sp = std::sin(phi), cp = std::cos(phi);
        ls.wi = xf_vec(L.l2w, V3(st * cp, st * sp, ct));
        ls.pdf = st == 0.0f ? 0.0f : map_pdf / (2.0f * PI * PI * st);
        ls.radiance = mip_trilinear(L.map, uv[0], uv[1], 0.0f);
        ls.p0 = it;
        ls.p0.surface = false;
        ls.p1 = Interaction();
        ls.p1.p = it.p + ls.wi * (2.0f * L.radius);
        ls.p1.time = it.time;
        ls.vis = true;
        return ls;
    }
    float pdf_area;
    Interaction pit = prim < s.ntri ? tri_sample(s, prim, u0, u1, &pdf_area)
                      : prim < s.ntri + s.nsph ? sphere_sample(s.sph[prim - s.ntri], u0, u1, mode, &pdf_area)
                                               : quadric_sample(s.quads[prim - s.ntri - s.nsph], u0, u1, mode, &pdf_area);
    V3 wi = pit.p - it.p;
    float pdf;
    if (length_squared(wi) == 0.0f) pdf = 0.0f;
    else {
        wi = normalize(wi);
        // F13: REF overwrites the area pdf with dist^2/|cos| (shape.rs:31-32); PBRT multiplies
        float conv = distance_squared(it.p, pit.p) / abs_dot(pit.n, -wi);
        pdf = mode == REF ? conv : pdf_area * conv;
        if (std::isinf(pdf)) pdf = 0.0f;
    }
    if (pdf == 0.0f || length_squared(pit.p - it.p) == 0.0f) return ls;
    ls.wi = normalize(pit.p - it.p);
    // F12: REF evaluates the emission toward +wi (diffuse.rs:67); PBRT toward -wi
    ls.radiance = emission(s.emis[s.prim_emission[prim]], pit.n, mode == REF ? ls.wi : -ls.wi);
    ls.pdf = pdf;
    ls.p0 = it;
    ls.p0.surface = false;
    ls.p1 = pit;
    ls.vis = true;
    return ls;
}
static float light_point_pdf(const Scene& s, int64_t prim, const Interaction& it, V3 wi, Mode mode) {  // shape.rs:40-57
    if (prim == LIGHT_INF) {  // InfiniteAreaLight::point_pdf (infinite.rs:155-169)
        V3 w = xf_vec(s.inf.w2l, wi);
        float theta = sph_theta(w), phi = sph_phi(w);
        float st = std::sin(theta);
        if (st == 0.0f) return 0.0f;
        return d2_pdf(s.inf, phi * (1.0f / (2.0f * PI)), theta * (1.0f / PI), mode) / (2.0f * PI * PI * st);
    }
    Ray ray = spawn_ray(it, wi, mode);
    float t;
    Interaction iit;
    float area;
    if (prim < s.ntri) {
        if (!tri_intersect(s, prim, ray, &t, &iit, false)) return 0.0f;
        area = tri_area(s, prim);
    } else if (prim < s.ntri + s.nsph) {
        const Sphere& sp = s.sph[prim - s.ntri];
        if (mode == REF) {  // F20: Sphere::pdf_from_it (sphere.rs:357-373)
            V3 center = xf_point(sp.o2w, V3(0.0f, 0.0f, 0.0f));
            V3 origin = offset_ray_origin(it.p, it.p_err, it.n, center - it.p);
            if (!(distance_squared(origin, center) <= sp.radius * sp.radius)) {
                float sin2 = sp.radius * sp.radius / distance_squared(it.p, center);
                float cos_max = std::sqrt(rmax(0.0f, 1.0f - sin2));
                return 1.0f / (2.0f * PI * (1.0f - cos_max));  // uniform_cone_pdf
            }
        }
        if (!sphere_intersect(sp, ray, &t, &iit, false)) return 0.0f;
        area = sphere_area(sp);
    } else {
        const Quadric& q = s.quads[prim - s.ntri - s.nsph];
        if (!quadric_intersect(q, ray, &t, &iit, false)) return 0.0f;
        area = quadric_area(q);
    }
    float pdf = distance_squared(it.p, iit.p) / (abs_dot(iit.n, -wi) * area);
    if (std::isinf(pdf)) pdf = 0.0f;
    return pdf;
}
static float power_heuristic(float nf, float fpdf, float ng, float gpdf) {  // sampling.rs:248-252
    float f = nf * fpdf, g = ng * gpdf;
    return (f * f) / (f * f + g * g);
}

// estimate_direct (src/base/integrator.rs:330-437)
static RGB estimate_direct(const Scene& s, const Interaction& it, const BSDF& bsdf, int64_t light_prim, float us0,
                           float us1, float ul0, float ul1, Mode mode, Counters* cnt) {
    const uint8_t flags = BSDF_ALL & ~BSDF_SPECULAR;
    RGB out;
    LightSample ls = light_sample_point(s, light_prim, it, ul0, ul1, mode);
    float scattering_pdf = 0.0f;
    if (ls.pdf > 0.0f && !ls.radiance.is_black()) {
        RGB f = bsdf.f(it.wo, ls.wi, flags, mode) * abs_dot(ls.wi, it.shading_n);
        scattering_pdf = bsdf.pdf(it.wo, ls.wi, flags, mode);
        if (!f.is_black()) {
            if (cnt) cnt->shadow_rays++;
            if (scene_intersect_test(s, spawn_ray_to_it(ls.p0, ls.p1), cnt)) ls.radiance = RGB();
            if (!ls.radiance.is_black()) {
                float w = power_heuristic(1.0f, ls.pdf, 1.0f, scattering_pdf);
                out = out + f * ls.radiance * w / ls.pdf;
            }
        }
    }
    // BSDF sampling half
    BxSample bs = bsdf.sample(it.wo, us0, us1, flags, mode);
    RGB f = bs.f * abs_dot(bs.wi, it.shading_n);
    bool sampled_specular = (bs.sampled_type & BSDF_SPECULAR) != 0;
    if (mode == REF) {
        // F2: ray along the LIGHT sample direction, pdf and weight from the light half, any emitter
        if (!f.is_black() && scattering_pdf > 0.0f) {
            float w = 1.0f;
            if (!sampled_specular) {
                float lpdf = light_point_pdf(s, light_prim, it, ls.wi, mode);
                if (lpdf == 0.0f) return out;
                w = power_heuristic(1.0f, scattering_pdf, 1.0f, lpdf);
            }
            Interaction lit;
            Ray ray = spawn_ray(it, ls.wi, mode);
            if (cnt) cnt->ext_rays++;
            RGB rad;
            if (scene_intersect(s, ray, &lit, cnt)) {
                if (s.prim_emission[lit.prim] >= 0) rad = emitted_radiance(s, lit, -ls.wi);
            } else if (light_prim == LIGHT_INF) {
                rad = inf_radiance(s, ray.d);  // light.radiance(&ray)
            }
            if (!rad.is_black()) out = out + f * rad * w / scattering_pdf;
        }
    } else {
        float spdf = bs.pdf;
        if (!f.is_black() && spdf > 0.0f) {
            float w = 1.0f;
            if (!sampled_specular) {
                float lpdf = light_point_pdf(s, light_prim, it, bs.wi, mode);
                if (lpdf == 0.0f) return out;
                w = power_heuristic(1.0f, spdf, 1.0f, lpdf);
            }
            Interaction lit;
            Ray ray = spawn_ray(it, bs.wi, mode);
            if (cnt) cnt->ext_rays++;
            RGB li;
            if (scene_intersect(s, ray, &lit, cnt)) {
                if (lit.prim == light_prim) li = emitted_radiance(s, lit, -bs.wi);
            } else if (light_prim == LIGHT_INF) {
                li = inf_radiance(s, ray.d);
            }
            if (!li.is_black()) out = out + f * li * w / spdf;
        }
    }
    return out;
}

// ---------------------------------------------------------------- camera (perspective.rs)
struct Camera {
    Transform raster_to_camera, camera_to_world;
    int w, h;
    float lens_radius = 0.0f, focal_distance = 1e6f;
    explicit Camera(const bg_camera& c) {  // perspective.rs:49-113
        w = (int)c.width;
        h = (int)c.height;
        lens_radius = c.lens_radius;
        focal_distance = c.focal_distance;
        float rx = (float)c.width, ry = (float)c.height;
        Transform c2s = t_perspective(c.fov_deg, c.near_plane, c.far_plane);
        float sminx, smaxx, sminy, smaxy;
        float frame = rx / ry;
        if (frame > 1.0f) { sminx = -frame; smaxx = frame; sminy = -1.0f; smaxy = 1.0f; }
        else { sminx = -1.0f; smaxx = 1.0f; sminy = -1.0f / frame; smaxy = 1.0f / frame; }
        Transform s2r = t_mul(t_mul(t_scale(rx, ry, 1.0f),
                                    t_scale(1.0f / (smaxx - sminx), 1.0f / (sminy - smaxy), 1.0f)),
                              t_translate(V3(-sminx, -smaxy, 0.0f)));
        Transform r2s = t_inverse(s2r);
        raster_to_camera = t_mul(t_inverse(c2s), r2s);
        camera_to_world = t_look_at(V3(c.position[0], c.position[1], c.position[2]),
                                    V3(c.look_at[0], c.look_at[1], c.look_at[2]), V3(c.up[0], c.up[1], c.up[2]));
    }
    // The lens point and the direction through the plane of focus (perspective.rs:127-139).
    void thin_lens(V3 d, float lu0, float lu1, V3* o, V3* dir) const {
        float ly;
        float lx = concentric_sample_disk(lu0, lu1, &ly).x;
        lx = lens_radius * lx;
        ly = lens_radius * ly;
        float t = focal_distance / d.z;
        V3 focus(0.0f + d.x * t, 0.0f + d.y * t, 0.0f + d.z * t);  // Ray::at from the origin
        *o = V3(lx, ly, 0.0f);
        *dir = normalize(focus - *o);
    }
    Ray generate_ray(float fx, float fy, float tu, float lu0 = 0.5f, float lu1 = 0.5f) const {  // perspective.rs:117-175
        V3 cp = xf_point(raster_to_camera, V3(fx, fy, 0.0f));
        Ray r{V3(0, 0, 0), normalize(cp), INFINITY, 0.0f};
        if (lens_radius > 0.0f) thin_lens(r.d, lu0, lu1, &r.o, &r.d);
        r.time = (1.0f - tu) * 0.0f + tu * 1.0f;  // lerp(time, 0, 1), math.rs:7-9
        return xf_ray(camera_to_world, r);
    }
    // The same ray's differentials (perspective.rs:141-170), moved to world space by Ray::transform
    // (ray.rs:66-73) and scaled by Ray::scale_differentials (ray.rs:41-48).
    RayDifferential differentials(float fx, float fy, const Ray& world_ray, float scale, float lu0 = 0.5f,
                                  float lu1 = 0.5f) const {
        V3 origin = xf_point(raster_to_camera, V3(0, 0, 0));
        V3 dx_camera = xf_point(raster_to_camera, V3(1, 0, 0)) - origin;  // perspective.rs:86-89
        V3 dy_camera = xf_point(raster_to_camera, V3(0, 1, 0)) - origin;
        V3 cp = xf_point(raster_to_camera, V3(fx, fy, 0.0f));
        V3 dx = normalize(cp + dx_camera), dy = normalize(cp + dy_camera);
        V3 ox(0, 0, 0), oy(0, 0, 0);
        if (lens_radius > 0.0f) {  // perspective.rs:141-157
            thin_lens(dx, lu0, lu1, &ox, &dx);
            thin_lens(dy, lu0, lu1, &oy, &dy);
        }
        RayDifferential d;
        d.has = true;
        d.rxo = xf_point(camera_to_world, ox);
        d.ryo = xf_point(camera_to_world, oy);
        d.rxd = xf_vec(camera_to_world, dx);
        d.ryd = xf_vec(camera_to_world, dy);
        const V3 o = world_ray.o, dd = world_ray.d;
        d.rxo = o + (d.rxo - o) * scale;
        d.ryo = o + (d.ryo - o) * scale;
        d.rxd = dd + (d.rxd - dd) * scale;
        d.ryd = dd + (d.ryd - dd) * scale;
        return d;
    }
};

// ---------------------------------------------------------------- PathIntegrator::radiance
// src/integrators/path.rs:51-146
// rd0: the camera ray's differentials; REF keeps them on every bounce (the ray never re-spawns,
// F1), PBRT has them at the first hit only (spawn_ray drops them).
static RGB radiance(const Scene& s, Ray ray, const CounterRng& rng, uint32_t max_depth, float rr_threshold,
                    Mode mode, Counters* cnt, const RayDifferential& rd0 = RayDifferential(),
                    const Strat& sp = Strat()) {
    SamplerCalls calls{sp, mode == REF, rng, 1u, 2u};  // after the camera sample's calls
    RGB out, beta(1.0f);
    bool specular_bounce = false;
    float eta_scale = 1.0f;
    uint32_t bounces = 0;
    for (;;) {
        Interaction it;
        if (cnt) cnt->ext_rays++;
        bool hit = scene_intersect(s, ray, &it, cnt);
        if (bounces == 0 || specular_bounce) {
            if (hit) out = out + beta * emitted_radiance(s, it, -ray.d);
            else out = out + beta * escaped_radiance(s, ray.d);  // path.rs:81-83
        }
        if (!hit || bounces >= max_depth) break;
        compute_differentials(&it, (mode == REF || bounces == 0) ? rd0 : RayDifferential());
        BSDF bsdf = make_bsdf(s, it, mode);
        const uint32_t base = DIM_BOUNCE0 + DIMS_PER_BOUNCE * bounces;
        if (bsdf.num_components(BSDF_ALL & ~BSDF_SPECULAR) > 0 && !s.light_prims.empty()) {
            // uniform_sample_one_light (integrator.rs:309-328)
            float count = (float)s.light_prims.size();
            const float upick = calls.get_1d(rng.u(base + BD_LIGHT));
            float ul0 = rng.u(base + BD_ULIGHT), ul1 = rng.u(base + BD_ULIGHT + 1);
            calls.get_2d(&ul0, &ul1);
            float us0 = rng.u(base + BD_USCAT), us1 = rng.u(base + BD_USCAT + 1);
            calls.get_2d(&us0, &us1);
            size_t li = (size_t)rmin(upick * count, count - 1.0f);
            float light_pdf = 1.0f / count;
            RGB ld = estimate_direct(s, it, bsdf, s.light_prims[li], us0, us1, ul0, ul1, mode, cnt);
            out = out + beta * (ld / light_pdf);
        }
        V3 wo = -ray.d;
        float ub0 = rng.u(base + BD_BSDF), ub1 = rng.u(base + BD_BSDF + 1);
        calls.get_2d(&ub0, &ub1);
        BxSample bs = bsdf.sample(wo, ub0, ub1, BSDF_ALL, mode);
        if (bs.f.is_black() || bs.pdf == 0.0f) break;
        beta = beta * (bs.f * abs_dot(bs.wi, it.shading_n) / bs.pdf);
        specular_bounce = (bs.sampled_type & BSDF_SPECULAR) != 0;
        if ((bs.sampled_type & BSDF_SPECULAR) && (bs.sampled_type & BSDF_TRANSMISSION)) {
            float eta = bsdf.eta;
            eta_scale *= dot(wo, it.n) > 0.0f ? eta * eta : 1.0f / (eta * eta);
        }
        // F1: REF keeps re-intersecting the same camera ray (t_max already at the hit);
        // PBRT spawns the next ray along the sampled direction.
        if (mode == PBRT) ray = spawn_ray(it, bs.wi, mode);
        RGB rr_beta = beta * eta_scale;
        if (rr_beta.max_component_value() < rr_threshold && bounces > 3) {
            float q = rmax(1.0f - rr_beta.max_component_value(), 0.5f);
            if (calls.get_1d(rng.u(base + BD_RR)) < q) break;
            beta = beta / (1.0f - q);
        }
        bounces += 1;
    }
    return out;
}

// ---------------------------------------------------------------- Whitted / DirectLighting
// WhittedIntegrator::radiance (src/integrators/whitted.rs:147-201), DirectLightingIntegrator::
// radiance (src/integrators/direct.rs:65-111) with specular_reflect / specular_transmit and
// uniform_sample_all_lights (src/base/integrator.rs:143-307), recursively as the reference.
// kind 1 Whitted, 2 direct with UniformSampleAll, 3 direct with UniformSampleOne.  Random numbers:
// stream = node - 1 of the ray tree (root 1, reflection 2k, transmission 2k + 1); dims 8-9
// reflection, 10-11 transmission, lights from 12 (Whitted 12 + 2j; all lights 12 + 4j u_light,
// +2 u_scattering; one light: pick 12, u_light 13-14, u_scattering 15-16).
static RGB tree_radiance(const Scene& s, Ray ray, const RayDifferential& rd, CounterRng rng, uint32_t node,
                         uint32_t depth, uint32_t max_depth, int kind, Mode mode, Counters* cnt) {
    RGB out;
    Interaction it;
    if (cnt) cnt->ext_rays++;
    if (!scene_intersect(s, ray, &it, cnt)) return escaped_radiance(s, ray.d);  // whitted.rs:45-51
    rng.stream = node - 1;
    compute_differentials(&it, rd);
    BSDF bsdf = make_bsdf(s, it, mode, false);  // allow_multiple_lobes = false
    out = out + emitted_radiance(s, it, it.wo);
    const size_t nl = s.light_prims.size();
    if (nl > 0) {
        if (kind == 1) {
            for (size_t j = 0; j < nl; ++j) {
                LightSample ls = light_sample_point(s, s.light_prims[j], it, rng.u(12 + 2 * (uint32_t)j),
                                                    rng.u(13 + 2 * (uint32_t)j), mode);
                if (ls.radiance.is_black() || ls.pdf == 0.0f) continue;
                RGB f = bsdf.f(it.wo, ls.wi, BSDF_ALL, mode);
                if (!ls.vis || f.is_black()) continue;
                if (cnt) cnt->shadow_rays++;
                if (scene_intersect_test(s, spawn_ray_to_it(ls.p0, ls.p1), cnt)) continue;
                out = out + f * ls.radiance * abs_dot(ls.wi, it.shading_n) / ls.pdf;
            }
        } else if (kind == 2) {
            for (size_t j = 0; j < nl; ++j) {
                const uint32_t b = 12 + 4 * (uint32_t)j;
                RGB d = estimate_direct(s, it, bsdf, s.light_prims[j], rng.u(b + 2), rng.u(b + 3), rng.u(b), rng.u(b + 1),
                                        mode, cnt);
                out = out + d / 1.0f;
            }
        } else {
            float count = (float)nl;
            size_t li = (size_t)rmin(rng.u(12) * count, count - 1.0f);
            RGB d = estimate_direct(s, it, bsdf, s.light_prims[li], rng.u(15), rng.u(16), rng.u(13), rng.u(14), mode, cnt);
            out = out + d / (1.0f / count);
        }
    }
    if (depth + 1 < max_depth) {
        for (int k = 0; k < 2; ++k) {  // specular_reflect, then specular_transmit
            const uint8_t type = k == 0 ? (BSDF_REFLECTION | BSDF_SPECULAR) : (BSDF_TRANSMISSION | BSDF_SPECULAR);
            BxSample bs = bsdf.sample(it.wo, rng.u(8 + 2 * k), rng.u(9 + 2 * k), type, mode);
            V3 normal = it.shading_n;
            if (!(bs.pdf > 0.0f) || bs.f.is_black() || abs_dot(bs.wi, normal) == 0.0f) continue;
            Ray child = spawn_ray(it, bs.wi, mode);
            RayDifferential crd;
            if (rd.has) {
                crd.has = true;
                crd.rxo = it.p + it.dpdx;
                crd.ryo = it.p + it.dpdy;
                V3 dndx = it.shading_dndu * it.dudx + it.shading_dndv * it.dvdx;
                V3 dndy = it.shading_dndu * it.dudy + it.shading_dndv * it.dvdy;
                const V3 wo = it.wo;
                if (k == 0) {
                    V3 dwodx = -rd.rxd - wo, dwody = -rd.ryd - wo;
                    float ddndx = dot(dwodx, normal) + dot(wo, dndx);
                    float ddndy = dot(dwody, normal) + dot(wo, dndy);
                    crd.rxd = bs.wi - dwodx + 2.0f * (dot(wo, normal) * dndx + ddndx * normal);
                    crd.ryd = bs.wi - dwody + 2.0f * (dot(wo, normal) * dndy + ddndy * normal);
                } else {
                    float eta = 1.0f / bsdf.eta;
                    if (dot(wo, normal) < 0.0f) {
                        eta = 1.0f / eta;
                        normal = -normal;
                        dndx = -dndx;
                        dndy = -dndy;
                    }
                    V3 dwodx = -rd.rxd - wo, dwody = -rd.ryd - wo;
                    float ddndx = dot(dwodx, normal) + dot(wo, dndx);
                    float ddndy = dot(dwody, normal) + dot(wo, dndy);
                    float mu = eta * dot(wo, normal) - abs_dot(bs.wi, normal);
                    float dmudx = (eta - (eta * eta * dot(wo, normal)) / abs_dot(bs.wi, normal)) * ddndx;
                    float dmudy = (eta - (eta * eta * dot(wo, normal)) / abs_dot(bs.wi, normal)) * ddndy;
                    crd.rxd = bs.wi - eta * dwodx + (mu * dndx + dmudx * normal);
                    crd.ryd = bs.wi - eta * dwody + (mu * dndy + dmudy * normal);
                }
            }
            RGB li = tree_radiance(s, child, crd, rng, 2 * node + (uint32_t)k, depth + 1, max_depth, kind, mode, cnt);
            out = out + bs.f * li * abs_dot(bs.wi, normal) / bs.pdf;
        }
    }
    return out;
}

}  // namespace orc

using namespace orc;

// ================================================================= C API (ctypes)
extern "C" {

void* orc_scene_create(const float* tri_xyz, int64_t ntri, const uint32_t* tri_mat, const int32_t* tri_light,
                       const bg_sphere* sph, int64_t nsph, const bg_material* mats, int32_t nmat,
                       const bg_area_light* emis, int32_t nemis, int32_t bvh_fixed, const bg_quadric* quads,
                       int64_t nquad) {
    Scene* s = new Scene();
    s->ntri = ntri;
    s->nsph = nsph;
    s->nquad = nquad;
    s->pos.resize(3 * ntri);
    for (int64_t i = 0; i < 3 * ntri; ++i) s->pos[i] = V3(tri_xyz[3 * i], tri_xyz[3 * i + 1], tri_xyz[3 * i + 2]);
    s->tri_mat.assign(tri_mat, tri_mat + ntri);
    s->mats.assign(mats, mats + nmat);
    s->emis.assign(emis, emis + nemis);
    s->prim_emission.assign(ntri + nsph + nquad, -1);
    s->prim_light.assign(ntri + nsph + nquad, -1);
    for (int64_t i = 0; i < ntri; ++i) {
        if (tri_light && tri_light[i] >= 0) {
            s->prim_emission[i] = tri_light[i];
            s->prim_light[i] = (int32_t)s->light_prims.size();
            s->light_prims.push_back(i);
        }
    }
    for (int64_t i = 0; i < nsph; ++i) {
        Sphere sp;
        V3 c(sph[i].center[0], sph[i].center[1], sph[i].center[2]);
        sp.o2w = t_translate(c);
        sp.w2o = is_identity(sp.o2w) ? sp.o2w : t_inverse(sp.o2w);
        float r = sph[i].radius;
        sp.radius = r;
        sp.z_min = rclamp(rmin(-r, r), -r, r);
        sp.z_max = rclamp(rmax(-r, r), -r, r);
        sp.theta_min = std::acos(rclamp(rmin(-r, r) / r, -1.0f, 1.0f));
        sp.theta_max = std::acos(rclamp(rmax(-r, r) / r, -1.0f, 1.0f));
        sp.phi_max = rclamp(360.0f, 0.0f, 360.0f) * (PI / 180.0f);
        sp.mat = sph[i].material_id;
        s->sph.push_back(sp);
        if (sph[i].light_id >= 0) {  // DiffuseAreaLight on the sphere
            s->prim_emission[ntri + i] = sph[i].light_id;
            s->prim_light[ntri + i] = (int32_t)s->light_prims.size();
            s->light_prims.push_back(ntri + i);
        }
    }
    for (int64_t i = 0; i < nquad; ++i) {
        const bg_quadric& g = quads[i];
        Quadric q;
        q.kind = (int)g.kind;
        q.o2w.m = Mat4::identity();
        q.w2o.m = Mat4::identity();
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 4; ++c) {
                q.o2w.m.m[r][c] = g.object_to_world[4 * r + c];
                q.w2o.m.m[r][c] = g.world_to_object[4 * r + c];
            }
        q.o2w.mi = q.w2o.m;
        q.w2o.mi = q.o2w.m;
        if (is_identity(q.o2w)) q.w2o = q.o2w;  // cylinder.rs:37-41
        const auto& m = q.o2w.m.m;  // Transform::swaps_handedness (transform.rs:212-218)
        float det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                    m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
        q.swaps = det < 0.0f;
        q.reverse = g.reverse_orientation != 0;
        q.radius = g.radius;
        q.inner = g.inner_radius;
        q.z_min = rmin(g.z_min, g.z_max);
        q.z_max = rmax(g.z_min, g.z_max);
        q.height = g.height;
        q.phi_max = rclamp(g.phi_max_deg, 0.0f, 360.0f) * (PI / 180.0f);
        q.mat = g.material_id;
        s->quads.push_back(q);
        if (g.light_id >= 0) {
            s->prim_emission[ntri + nsph + i] = g.light_id;
            s->prim_light[ntri + nsph + i] = (int32_t)s->light_prims.size();
            s->light_prims.push_back(ntri + nsph + i);
        }
    }
    build_bvh(*s, bvh_fixed != 0);
    return s;
}

// Triangle mesh attributes (bg_scene_add_triangle_mesh): normals 9 floats per triangle (rows
// where has_normals[i] == 0 are ignored), uvs 6 floats per triangle or NULL, flags per triangle
// (BG_TRI_* bits) or NULL.
void orc_scene_set_tri_attrs(void* p, const float* normals, const uint8_t* has_normals, const float* uvs,
                             const uint8_t* flags) {
    Scene& s = *(Scene*)p;
    s.tri_flags.assign(s.ntri, 0);
    s.tri_n.assign(3 * s.ntri, V3(0, 0, 0));
    for (int64_t i = 0; i < s.ntri; ++i) {
        uint8_t f = 0;
        if (flags) {
            if (flags[i] & BG_TRI_REVERSE_ORIENTATION) f |= TA_REVERSE;
            if (flags[i] & BG_TRI_SWAPS_HANDEDNESS) f |= TA_SWAPS;
        }
        if (normals && (!has_normals || has_normals[i])) {
            f |= TA_NORMALS;
            for (int k = 0; k < 3; ++k)
                s.tri_n[3 * i + k] = V3(normals[9 * i + 3 * k], normals[9 * i + 3 * k + 1], normals[9 * i + 3 * k + 2]);
        }
        s.tri_flags[i] = f;
    }
    if (uvs) s.tri_uv.assign(uvs, uvs + 6 * s.ntri);
    else s.tri_uv.clear();
}
// Appends a texture (bg_texture); materials refer to it as (returned id) + 1.
int32_t orc_scene_add_texture(void* p, const bg_texture* t) {
    Scene& s = *(Scene*)p;
    Texture x;
    x.kind = t->kind;
    x.wrap = t->wrap;
    x.mapping = t->mapping;
    x.su = t->uv_scale[0];
    x.sv = t->uv_scale[1];
    x.du = t->uv_delta[0];
    x.dv = t->uv_delta[1];
    x.w2t.m = Mat4::identity();
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) x.w2t.m.m[r][c] = t->world_to_texture[4 * r + c];
    x.w2t.mi = mat_inverse(x.w2t.m);
    x.vs = V3(t->vs[0], t->vs[1], t->vs[2]);
    x.vt = V3(t->vt[0], t->vt[1], t->vt[2]);
    x.ds = t->ds;
    x.dt = t->dt;
    if (t->kind == BG_TEXTURE_IMAGE) {
        Image img;
        img.w = (int)t->width;
        img.h = (int)t->height;
        img.px.assign(t->rgb, t->rgb + (size_t)t->width * t->height * 3);
        x.pyramid = generate_pyramid(std::move(img));
    }
    s.tex.push_back(std::move(x));
    return (int32_t)s.tex.size() - 1;
}

// InfiniteAreaLight::new (infinite.rs:38-80) with the scene's BVH bounds as the world bounds; the
// light joins the end of the light list.
int32_t orc_scene_add_infinite_light(void* p, const bg_infinite_light* l) {
    Scene& s = *(Scene*)p;
    if (s.has_inf) return -1;
    InfiniteLight& L = s.inf;
    L.map.kind = BG_TEXTURE_IMAGE;
    L.map.wrap = BG_WRAP_REPEAT;
    Image img;
    img.w = (int)l->width;
    img.h = (int)l->height;
    img.px.assign(l->rgb, l->rgb + (size_t)l->width * l->height * 3);
    for (size_t i = 0; i < img.px.size(); ++i) img.px[i] *= l->intensity[i % 3];  // Image::scale
    L.map.pyramid = generate_pyramid(std::move(img));
    L.nu = 2 * l->width;
    L.nv = 2 * l->height;
    const float fwidth = 0.5f / (float)std::min(L.nu, L.nv);
    L.func.assign((size_t)L.nu * L.nv, 0.0f);
    for (uint32_t v = 0; v < L.nv; ++v) {
        float vp = ((float)v + 0.5f) / (float)L.nv;
        float sin_theta = std::sin(PI * ((float)v + 0.5f) / (float)L.nv);
        for (uint32_t u = 0; u < L.nu; ++u) {
            float up = ((float)u + 0.5f) / (float)L.nu;
            RGB c = mip_trilinear(L.map, up, vp, fwidth);
            L.func[(size_t)v * L.nu + u] = c.y() * sin_theta;  // RGBSpectrum::y
        }
    }
    // Distribution1D::new (sampling.rs:22-47) for each row, then the marginal
    auto build = [](const float* f, uint32_t n, float* cdf) {
        cdf[0] = 0.0f;
        for (uint32_t i = 1; i <= n; ++i) cdf[i] = cdf[i - 1] + f[i - 1] / (float)n;
        float integral = cdf[n];
        for (uint32_t i = 1; i <= n; ++i) cdf[i] = integral == 0.0f ? (float)i / (float)n : cdf[i] / integral;
        return integral;
    };
    L.cond_cdf.assign((size_t)L.nv * (L.nu + 1), 0.0f);
    L.cond_int.assign(L.nv, 0.0f);
    for (uint32_t v = 0; v < L.nv; ++v)
        L.cond_int[v] = build(&L.func[(size_t)v * L.nu], L.nu, &L.cond_cdf[(size_t)v * (L.nu + 1)]);
    L.marg_cdf.assign(L.nv + 1, 0.0f);
    L.marg_int = build(L.cond_int.data(), L.nv, L.marg_cdf.data());
    L.l2w.m = Mat4::identity();
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) L.l2w.m.m[r][c] = l->light_to_world[4 * r + c];
    L.l2w.mi = mat_inverse(L.l2w.m);
    L.w2l = t_inverse(L.l2w);
    // Bounds3::bounding_sphere (bounds3.rs:208-215) of the BVH's root bounds
    Bounds3 b = s.nodes.empty() ? Bounds3() : s.nodes[0].b;
    V3 c = (b.mn + b.mx) * (1.0f / 2.0f);
    bool inside = c.x >= b.mn.x && c.x <= b.mx.x && c.y >= b.mn.y && c.y <= b.mx.y && c.z >= b.mn.z && c.z <= b.mx.z;
    L.center = c;
    L.radius = inside ? length(c - b.mx) : 0.0f;
    s.has_inf = true;
    s.light_prims.push_back(LIGHT_INF);
    return 0;
}

// The stratified sampler's value for stratified dimension k (is2d: get_2d, else get_1d) of
// (pixel, sample) under the render options; out[1] = 0 for get_1d.  -1 when the options are not
// a stratified sampler.
int32_t orc_strat_sample(const bg_render_opts* o, uint32_t pixel, uint32_t sample, uint32_t k, int32_t is2d,
                         float* out) {
    if (o->sampler != BG_SAMPLER_STRATIFIED || o->x_pixel_samples * o->y_pixel_samples == 0) return -1;
    Strat sp;
    sp.dims = o->sampled_dimensions;
    sp.nx = o->x_pixel_samples;
    sp.ny = o->y_pixel_samples;
    sp.jitter = o->jitter_samples;
    CounterRng rng;
    rng.pixel = pixel;
    rng.sample = sample;
    rng.seed = o->seed;
    const bool ref = o->mode == BG_MODE_REF_COMPAT;
    if (is2d) {
        strat_2d(sp, ref, rng, k, &out[0], &out[1]);
    } else {
        out[0] = strat_1d(sp, ref, rng, k);
        out[1] = 0.0f;
    }
    return 0;
}

void orc_scene_destroy(void* p) { delete (Scene*)p; }
int64_t orc_bvh_nodes(void* p) { return (int64_t)((Scene*)p)->nodes.size(); }
int64_t orc_num_lights(void* p) { return (int64_t)((Scene*)p)->light_prims.size(); }

static void parallel_for(int64_t n, int threads, const std::function<void(int64_t, int)>& fn) {
    if (threads <= 1 || n <= 1) {
        for (int64_t i = 0; i < n; ++i) fn(i, 0);
        return;
    }
    std::atomic<int64_t> next(0);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&, t]() {
            for (;;) {
                int64_t i = next.fetch_add(1);
                if (i >= n) break;
                fn(i, t);
            }
        });
    for (auto& th : pool) th.join();
}

// Closest-hit / any-hit over a ray set; counters[0..1] = node visits, primitive tests.
void orc_trace(void* p, const bg_ray* rays, int64_t n, int32_t any_only, bg_hit* hits, uint8_t* occluded,
               int64_t* counters, int32_t threads) {
    const Scene& s = *(const Scene*)p;
    const int64_t chunk = 4096;
    int64_t nchunks = (n + chunk - 1) / chunk;
    int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
    std::vector<Counters> cs(nt);
    parallel_for(nchunks, nt, [&](int64_t c, int t) {
        Counters* cnt = counters ? &cs[t] : nullptr;
        for (int64_t i = c * chunk; i < std::min(n, (c + 1) * chunk); ++i) {
            Ray r{V3(rays[i].org[0], rays[i].org[1], rays[i].org[2]),
                  V3(rays[i].dir[0], rays[i].dir[1], rays[i].dir[2]), rays[i].tmax, 0.0f};
            if (any_only) {
                occluded[i] = scene_intersect_test(s, r, cnt) ? 1 : 0;
            } else {
                Interaction it;
                if (scene_intersect(s, r, &it, cnt)) { hits[i].prim = it.prim; hits[i].t = r.t_max; }
                else { hits[i].prim = -1; hits[i].t = INFINITY; }
            }
        }
    });
    if (counters) {
        Counters tot;
        for (auto& c : cs) tot.add(c);
        counters[0] = any_only ? tot.sh_visits : tot.ext_visits;
        counters[1] = any_only ? tot.sh_tests : tot.ext_tests;
    }
}

// Renders rows [y0, y1) with stride ystep (all columns), tile rows of 16 as parallel tasks
// (src/base/integrator.rs:35-133).  Outputs (each may be NULL): rgb (w*h*3, Film::write_image
// values for the rendered rows), sum / sumsq (w*h*3 doubles of the sanitized sample radiance).
// counters[0..6] = extension rays, shadow rays, ext visits, ext tests, shadow visits, shadow tests,
// zeroed samples (counted only when counters != NULL and count_traversal != 0 for 2..5).
int orc_render(void* p, const bg_camera* cam, const bg_render_opts* opts, int32_t y0, int32_t y1, int32_t ystep,
               int32_t threads, int32_t count_traversal, float* rgb, double* sum, double* sumsq, int64_t* counters) {
    const Scene& s = *(const Scene*)p;
    Camera camera(*cam);
    const int W = camera.w, H = camera.h;
    if (y0 < 0) y0 = 0;
    if (y1 > H) y1 = H;
    if (ystep < 1) ystep = 1;
    Mode mode = opts->mode == BG_MODE_PBRT ? PBRT : REF;
    int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
    const float diff_scale = 1.0f / std::sqrt((float)(opts->spp ? opts->spp : 1u));  // integrator.rs:80-82
    const int tree_kind = opts->integrator == BG_INTEGRATOR_WHITTED ? 1
                          : (opts->light_strategy == BG_LIGHT_UNIFORM_ALL ? 2 : 3);
    Strat sp;
    if (opts->sampler == BG_SAMPLER_STRATIFIED) {
        sp.dims = opts->sampled_dimensions;
        sp.nx = opts->x_pixel_samples;
        sp.ny = opts->y_pixel_samples;
        sp.jitter = opts->jitter_samples;
        if (sp.nx * sp.ny != opts->spp || sp.nx == 0) return -1;
    }
    const int TILE = 16;
    int ntx = (W + TILE - 1) / TILE, nty = (H + TILE - 1) / TILE;
    std::vector<Counters> cs(nt);
    parallel_for(nty, nt, [&](int64_t ty, int t) {
        Counters* cnt = (counters && count_traversal) ? &cs[t] : nullptr;
        Counters& cbase = cs[t];
        for (int tx = 0; tx < ntx; ++tx) {
            for (int y = (int)ty * TILE; y < std::min(H, (int)(ty + 1) * TILE); ++y) {
                if (y < y0 || y >= y1 || ((y - y0) % ystep) != 0) continue;
                for (int x = tx * TILE; x < std::min(W, (tx + 1) * TILE); ++x) {
                    RGB tile_sum;  // FilmTilePixel::contribution_sum (f32)
                    float wsum = 0.0f;
                    double s1[3] = {0, 0, 0}, s2[3] = {0, 0, 0};
                    CounterRng rng;
                    rng.pixel = (uint32_t)(y * W + x);
                    rng.seed = opts->seed;
                    for (uint32_t si = 0; si < opts->spp; ++si) {
                        rng.sample = opts->first_sample + si;
                        // Sampler::get_camera_sample: film get_2d, lens get_2d, time get_1d
                        float ux = rng.u(DIM_FILM), uy = rng.u(DIM_FILM + 1);
                        float lx = rng.u(DIM_LENS), ly = rng.u(DIM_LENS + 1);
                        float ut = rng.u(DIM_TIME);
                        if (sp.dims > 0) {
                            strat_2d(sp, mode == REF, rng, 0, &ux, &uy);
                            ut = strat_1d(sp, mode == REF, rng, 0);
                            if (sp.dims > 1) strat_2d(sp, mode == REF, rng, 1, &lx, &ly);
                        }
                        float fx = (float)x + ux, fy = (float)y + uy;
                        Ray ray = camera.generate_ray(fx, fy, ut, lx, ly);
                        RayDifferential rd;
                        if (!s.tex.empty()) rd = camera.differentials(fx, fy, ray, diff_scale, lx, ly);
                        Counters local;
                        Counters* cc = cnt ? cnt : (counters ? &local : nullptr);
                        RGB L = opts->integrator == BG_INTEGRATOR_PATH
                                    ? radiance(s, ray, rng, opts->max_depth, opts->rr_threshold, mode, cc, rd, sp)
                                    : tree_radiance(s, ray, rd, rng, 1, 0, opts->max_depth, tree_kind, mode, cc);
                        if (!cnt && counters) { cbase.ext_rays += local.ext_rays; cbase.shadow_rays += local.shadow_rays; }
                        // sanity checks (integrator.rs:91-117)
                        if (L.is_nan() || L.y() < -1e-5f || std::isinf(L.y())) {
                            L = RGB();
                            cbase.nan_samples++;
                        }
                        // FilmTile::add_sample with BoxFilter r=0.5: weight 1 to the sample's pixel
                        tile_sum = tile_sum + L * 1.0f * 1.0f;
                        wsum += 1.0f;
                        for (int c = 0; c < 3; ++c) { s1[c] += L.c[c]; s2[c] += (double)L.c[c] * L.c[c]; }
                    }
                    size_t pix = (size_t)y * W + x;
                    if (sum) for (int c = 0; c < 3; ++c) sum[3 * pix + c] = s1[c];
                    if (sumsq) for (int c = 0; c < 3; ++c) sumsq[3 * pix + c] = s2[c];
                    if (rgb) {
                        // merge_film_tile (rgb_to_xyz, film.rs:138-154) + write_image (film.rs:156-202)
                        float X = 0.412453f * tile_sum.c[0] + 0.357580f * tile_sum.c[1] + 0.180423f * tile_sum.c[2];
                        float Y = 0.212671f * tile_sum.c[0] + 0.715160f * tile_sum.c[1] + 0.072169f * tile_sum.c[2];
                        float Z = 0.019334f * tile_sum.c[0] + 0.119193f * tile_sum.c[1] + 0.950227f * tile_sum.c[2];
                        float r = 3.240479f * X - 1.537150f * Y - 0.498535f * Z;
                        float g = -0.969256f * X + 1.875991f * Y + 0.041556f * Z;
                        float b = 0.055648f * X - 0.204043f * Y + 1.057311f * Z;
                        if (wsum != 0.0f) {
                            float inv = 1.0f / wsum;
                            r = rmax(r * inv, 0.0f);
                            g = rmax(g * inv, 0.0f);
                            b = rmax(b * inv, 0.0f);
                        }
                        rgb[3 * pix] = r;
                        rgb[3 * pix + 1] = g;
                        rgb[3 * pix + 2] = b;
                    }
                }
            }
        }
    });
    if (counters) {
        Counters tot;
        for (auto& c : cs) tot.add(c);
        counters[0] = tot.ext_rays;
        counters[1] = tot.shadow_rays;
        counters[2] = tot.ext_visits;
        counters[3] = tot.ext_tests;
        counters[4] = tot.sh_visits;
        counters[5] = tot.sh_tests;
        counters[6] = tot.nan_samples;
    }
    return 0;
}

// Unit probes used by the tests: one BSDF sample / eval for a material at a canonical frame.
// frame: ns = (0,0,1), ng = ns, ss = (1,0,0).  out[0..2] f, out[3] pdf, out[4..6] wi, out[7] type.
void orc_bsdf_sample(const bg_material* m, const float* wo, float u0, float u1, int32_t mode, float* out) {
    Scene s;
    s.ntri = 1;
    s.tri_mat.push_back(0);
    s.mats.push_back(*m);
    Interaction it;
    it.prim = 0;
    it.n = V3(0, 0, 1);
    it.shading_n = it.n;
    it.shading_dpdu = V3(1, 0, 0);
    BSDF b = make_bsdf(s, it, mode == 1 ? PBRT : REF);
    BxSample bs = b.sample(V3(wo[0], wo[1], wo[2]), u0, u1, BSDF_ALL, mode == 1 ? PBRT : REF);
    out[0] = bs.f.c[0]; out[1] = bs.f.c[1]; out[2] = bs.f.c[2]; out[3] = bs.pdf;
    out[4] = bs.wi.x; out[5] = bs.wi.y; out[6] = bs.wi.z; out[7] = (float)bs.sampled_type;
}
void orc_bsdf_eval(const bg_material* m, const float* wo, const float* wi, int32_t mode, float* out) {
    Scene s;
    s.ntri = 1;
    s.tri_mat.push_back(0);
    s.mats.push_back(*m);
    Interaction it;
    it.prim = 0;
    it.n = V3(0, 0, 1);
    it.shading_n = it.n;
    it.shading_dpdu = V3(1, 0, 0);
    Mode md = mode == 1 ? PBRT : REF;
    BSDF b = make_bsdf(s, it, md);
    RGB f = b.f(V3(wo[0], wo[1], wo[2]), V3(wi[0], wi[1], wi[2]), BSDF_ALL, md);
    out[0] = f.c[0]; out[1] = f.c[1]; out[2] = f.c[2];
    out[3] = b.pdf(V3(wo[0], wo[1], wo[2]), V3(wi[0], wi[1], wi[2]), BSDF_ALL, md);
}
// Raw Philox4x32-10 block (known-answer tests).
void orc_philox(const uint32_t* ctr_in, const uint32_t* key, uint32_t* out) {
    uint32_t c[4] = {ctr_in[0], ctr_in[1], ctr_in[2], ctr_in[3]};
    philox4x32_10(c, key[0], key[1]);
    for (int i = 0; i < 4; ++i) out[i] = c[i];
}
float orc_rng_uniform(uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t dim) {
    CounterRng r;
    r.seed = seed;
    r.pixel = pixel;
    r.sample = sample;
    return r.u(dim);
}
// Camera ray for a film sample (perspective.rs:117-175): out = ox oy oz dx dy dz.
void orc_camera_ray(const bg_camera* cam, float fx, float fy, float tu, float lu0, float lu1, float* out) {
    Camera c(*cam);
    Ray r = c.generate_ray(fx, fy, tu, lu0, lu1);
    out[0] = r.o.x; out[1] = r.o.y; out[2] = r.o.z; out[3] = r.d.x; out[4] = r.d.y; out[5] = r.d.z;
}

}  // extern "C"

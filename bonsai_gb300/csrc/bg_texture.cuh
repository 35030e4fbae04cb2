// bg_texture.cuh - ray differentials, texture mappings and MIPMap lookups on the device.
//
// Restates PerspectiveCamera's ray differentials (src/cameras/perspective.rs:141-170,
// src/geometries/ray.rs:41-48,50-76), Interaction::compute_differentials
// (src/base/interaction.rs:184-250), the TextureMapping2D implementations (src/base/texture.rs),
// ImageTexture / UVTexture (src/textures/{image,uv}.rs) and MIPMap::filter with its trilinear
// lookup (src/base/mipmap.rs, src/io/image.rs:130-159), in the reference's f32 operation order.
#pragma once
#include "bg_device.h"
#include "bg_math.cuh"
#include "bg_shapes.cuh"

namespace bg {

// RayDifferentials (ray.rs:7-13): offset rays one pixel right (x) and down (y).
struct RayDiff {
    V3 rxo, ryo, rxd, ryd;
};

// Screen-space derivatives of a shading point (SurfaceInteraction::dpdx .. dvdy).
struct SurfDiff {
    V3 dpdx, dpdy;
    float dudx, dvdx, dudy, dvdy;
};

// Everything a texture lookup reads at a shading point.
struct TexPoint {
    V3 p, n;
    SurfaceGeom g;
    SurfDiff d;
};

BG_D V3 xf_point_h(const float m[4][4], V3 p) {  // Point3::transform (point3.rs:51-69)
    float xp = m[0][0] * p.x + m[0][1] * p.y + m[0][2] * p.z + m[0][3];
    float yp = m[1][0] * p.x + m[1][1] * p.y + m[1][2] * p.z + m[1][3];
    float zp = m[2][0] * p.x + m[2][1] * p.y + m[2][2] * p.z + m[2][3];
    float wp = m[3][0] * p.x + m[3][1] * p.y + m[3][2] * p.z + m[3][3];
    if (wp == 1.0f) return v3(xp, yp, zp);
    return v3(xp, yp, zp) / wp;
}
BG_D V3 xf_vec_h(const float m[4][4], V3 v) {  // Vec3::transform (vec3.rs:35-44)
    return v3(m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z, m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z,
              m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z);
}

// The camera ray's differentials for film point (fx, fy), moved to world space by
// Ray::transform and scaled by Ray::scale_differentials(1 / sqrt(spp))
// (src/base/integrator.rs:76-82).  `r` is the camera ray of the same sample (camera_ray).
BG_D RayDiff camera_diff(const Camera& c, float fx, float fy, const Ray& r, float scale, float lu0 = 0.5f,
                         float lu1 = 0.5f) {
    V3 cp = xf_point_h(c.r2c, v3(fx, fy, 0.0f));
    V3 dx = normalize(cp + v3(c.dxc[0], c.dxc[1], c.dxc[2]));
    V3 dy = normalize(cp + v3(c.dyc[0], c.dyc[1], c.dyc[2]));
    V3 oxc = v3(0.0f, 0.0f, 0.0f), oyc = oxc;
    if (c.lens_radius > 0.0f) {  // perspective.rs:141-157: both offset rays through the same lens point
        thin_lens(c, dx, lu0, lu1, &oxc, &dx);
        thin_lens(c, dy, lu0, lu1, &oyc, &dy);
    }
    RayDiff d;
    d.rxo = xf_point_h(c.c2w, oxc);
    d.ryo = xf_point_h(c.c2w, oyc);
    d.rxd = xf_vec_h(c.c2w, dx);
    d.ryd = xf_vec_h(c.c2w, dy);
    d.rxo = r.o + (d.rxo - r.o) * scale;
    d.ryo = r.o + (d.ryo - r.o) * scale;
    d.rxd = r.d + (d.rxd - r.d) * scale;
    d.ryd = r.d + (d.ryd - r.d) * scale;
    return d;
}

// solve_linear_system_2x2 (src/base/math.rs:52-68)
BG_D bool solve2x2(float a00, float a01, float a10, float a11, float b0, float b1, float* x0, float* x1) {
    float det = a00 * a11 - a01 * a10;
    if (fabsf(det) < 1e-10f) return false;
    *x0 = (a11 * b0 - a01 * b1) / det;
    *x1 = (a00 * b1 - a10 * b0) / det;
    if (isnan(*x0) || isnan(*x1)) return false;
    return true;
}

// Interaction::compute_differentials (interaction.rs:184-250); rd == nullptr is a ray without
// differentials (every derivative 0).
BG_D SurfDiff compute_differentials(V3 p, V3 n, const SurfaceGeom& g, const RayDiff* rd) {
    SurfDiff s;
    s.dpdx = v3(0.0f, 0.0f, 0.0f);
    s.dpdy = v3(0.0f, 0.0f, 0.0f);
    s.dudx = s.dvdx = s.dudy = s.dvdy = 0.0f;
    if (!rd) return s;
    float d = dot(n, p);
    float tx = -(dot(n, rd->rxo) - d) / dot(n, rd->rxd);
    if (isinf(tx) || isnan(tx)) return s;
    V3 px = rd->rxo + tx * rd->rxd;
    float ty = -(dot(n, rd->ryo) - d) / dot(n, rd->ryd);
    if (isinf(ty) || isnan(ty)) return s;
    V3 py = rd->ryo + ty * rd->ryd;
    s.dpdx = px - p;
    s.dpdy = py - p;
    int d0, d1;
    if (fabsf(n.x) > fabsf(n.y) && fabsf(n.x) > fabsf(n.z)) {
        d0 = 1;
        d1 = 2;
    } else if (fabsf(n.y) > fabsf(n.z)) {
        d0 = 0;
        d1 = 2;
    } else {
        d0 = 0;
        d1 = 1;
    }
    float a00 = get(g.dpdu, d0), a01 = get(g.dpdv, d0), a10 = get(g.dpdu, d1), a11 = get(g.dpdv, d1);
    float bx0 = get(px, d0) - get(p, d0), bx1 = get(px, d1) - get(p, d1);
    float by0 = get(py, d0) - get(p, d0), by1 = get(py, d1) - get(p, d1);
    if (!solve2x2(a00, a01, a10, a11, bx0, bx1, &s.dudx, &s.dvdx)) {
        s.dudx = 0.0f;
        s.dvdx = 0.0f;
    }
    if (!solve2x2(a00, a01, a10, a11, by0, by1, &s.dudy, &s.dvdy)) {
        s.dudy = 0.0f;
        s.dvdy = 0.0f;
    }
    return s;
}

// ---- mappings (src/base/texture.rs:48-144)
BG_D V3 tex_xf_point(const TexInfo& t, V3 p) {  // affine world_to_texture: w is exactly 1
    const auto& m = t.m;
    return v3(m[0][0] * p.x + m[0][1] * p.y + m[0][2] * p.z + m[0][3],
              m[1][0] * p.x + m[1][1] * p.y + m[1][2] * p.z + m[1][3],
              m[2][0] * p.x + m[2][1] * p.y + m[2][2] * p.z + m[2][3]);
}
// SphericalMapping2D::sphere.  REF: phi scaled by 1/pi as written (texture.rs:53), PBRT: 1/(2 pi).
template <bool REF>
BG_D float2 map_sphere(const TexInfo& t, V3 p) {
    V3 v = normalize(tex_xf_point(t, p) - v3(0.0f, 0.0f, 0.0f));
    float theta = acosf(rclamp(v.z, -1.0f, 1.0f));
    float phi = atan2f(v.y, v.x);
    if (phi < 0.0f) phi = phi + 2.0f * PI;
    return make_float2(theta * (1.0f / PI), phi * (REF ? (1.0f / PI) : (1.0f / (2.0f * PI))));
}
BG_D float2 map_cylinder(const TexInfo& t, V3 p) {
    V3 v = normalize(tex_xf_point(t, p) - v3(0.0f, 0.0f, 0.0f));
    return make_float2((PI + atan2f(v.y, v.x)) * (1.0f / (2.0f * PI)), v.z);
}
BG_D float wrap_dst(float y) {  // "mapping discontinuity" handling of texture.rs:91-100
    if (y > 0.5f) return 1.0f - y;
    if (y < -0.5f) return -(y + 1.0f);
    return y;
}
template <bool REF>
BG_D float2 tex_map(const TexInfo& t, const TexPoint& tp, float2* dstdx, float2* dstdy) {
    if (t.mapping == MAP_UV) {
        *dstdx = make_float2(t.su * tp.d.dudx, t.sv * tp.d.dvdx);
        *dstdy = make_float2(t.su * tp.d.dudy, t.sv * tp.d.dvdy);
        return make_float2(t.su * tp.g.u + t.du, t.sv * tp.g.v + t.dv);
    }
    if (t.mapping == MAP_PLANAR) {
        V3 vs = v3(t.vs[0], t.vs[1], t.vs[2]), vt = v3(t.vt[0], t.vt[1], t.vt[2]);
        *dstdx = make_float2(dot(tp.d.dpdx, vs), dot(tp.d.dpdx, vt));
        *dstdy = make_float2(dot(tp.d.dpdy, vs), dot(tp.d.dpdy, vt));
        return make_float2(t.ds + dot(tp.p, vs), t.dt + dot(tp.p, vt));
    }
    const float DELTA = 0.1f;
    const bool sph = t.mapping == MAP_SPHERICAL;
    float2 st = sph ? map_sphere<REF>(t, tp.p) : map_cylinder(t, tp.p);
    float2 sx = sph ? map_sphere<REF>(t, tp.p + DELTA * tp.d.dpdx) : map_cylinder(t, tp.p + DELTA * tp.d.dpdx);
    float2 sy = sph ? map_sphere<REF>(t, tp.p + DELTA * tp.d.dpdy) : map_cylinder(t, tp.p + DELTA * tp.d.dpdy);
    *dstdx = make_float2((sx.x - st.x) / DELTA, wrap_dst((sx.y - st.y) / DELTA));
    *dstdy = make_float2((sy.x - st.x) / DELTA, wrap_dst((sy.y - st.y) / DELTA));
    return st;
}

// ---- MIPMap
// `as i32` of a float: saturating, NaN to 0.
BG_D int32_t sat_i32(float f) {
    if (isnan(f)) return 0;
    if (f >= 2147483648.0f) return 2147483647;
    if (f <= -2147483648.0f) return (-2147483647 - 1);
    return (int32_t)f;
}
// math::modulo (math.rs:43-50)
BG_D int32_t imod(int32_t a, int32_t b) {
    int32_t r = a - (a / b) * b;
    return r < 0 ? r + b : r;
}
// Image::get_channel with remap_pixel (image.rs:130-159), all three channels.
BG_D RGB texel(const Scene& sc, const TexInfo& t, int level, int32_t x, int32_t y) {
    const int32_t w = (int32_t)t.lw[level], h = (int32_t)t.lh[level];
    if (x < 0 || x >= w) {
        if (t.wrap == WRAP_BLACK) return rgb(0.0f);
        x = t.wrap == WRAP_REPEAT ? imod(x, w) : (x < 0 ? 0 : w - 1);
    }
    if (y < 0 || y >= h) {
        if (t.wrap == WRAP_BLACK) return rgb(0.0f);
        y = t.wrap == WRAP_REPEAT ? imod(y, h) : (y < 0 ? 0 : h - 1);
    }
    float4 v = __ldg(&sc.texels[t.loff[level] + (uint32_t)y * (uint32_t)w + (uint32_t)x]);
    return rgb(v.x, v.y, v.z);
}
BG_D int32_t wrap_add1(int32_t a) { return (int32_t)((uint32_t)a + 1u); }
// MIPMap::triangle (mipmap.rs:156-173): bilinear at one level.
BG_D RGB mip_bilerp(const Scene& sc, const TexInfo& t, int level, float2 st) {
    level = level < 0 ? 0 : (level > (int)t.nlevels - 1 ? (int)t.nlevels - 1 : level);
    float s = st.x * (float)t.lw[level] - 0.5f;
    float u = st.y * (float)t.lh[level] - 0.5f;
    float ds = s - floorf(s);
    float dt = u - floorf(u);
    int32_t s0 = sat_i32(floorf(s)), t0 = sat_i32(floorf(u));
    return (1.0f - ds) * (1.0f - dt) * texel(sc, t, level, s0, t0) +
           (1.0f - ds) * dt * texel(sc, t, level, s0, wrap_add1(t0)) +
           ds * (1.0f - dt) * texel(sc, t, level, wrap_add1(s0), t0) +
           ds * dt * texel(sc, t, level, wrap_add1(s0), wrap_add1(t0));
}
// MIPMap::filter + trilinear_filter (mipmap.rs:103-128)
BG_D RGB mip_filter(const Scene& sc, const TexInfo& t, float2 st, float2 d0, float2 d1) {
    float width = rmax(rmax(fabsf(d0.x), fabsf(d0.y)), rmax(fabsf(d1.x), fabsf(d1.y)));
    const float top = (float)(t.nlevels - 1);
    float level = top + log2f(rmax(width, 1e-8f));
    if (level < 0.0f) return mip_bilerp(sc, t, 0, st);
    if (level >= top) return texel(sc, t, (int)t.nlevels - 1, 0, 0);
    int il = (int)floorf(level);
    float f = level - floorf(level);
    RGB a = mip_bilerp(sc, t, il, st), b = mip_bilerp(sc, t, il + 1, st);
    return (1.0f - f) * a + f * b;
}

// Texture<RGBSpectrum>::evaluate for texture id `tid` (ImageTexture, image.rs:35-42; UVTexture,
// uv.rs:8-15).
template <bool REF>
BG_D RGB tex_eval(const Scene& sc, uint32_t tid, const TexPoint& tp) {
    const TexInfo& t = sc.tex[tid];
    float2 dx, dy;
    float2 st = tex_map<REF>(t, tp, &dx, &dy);
    if (t.kind == TEX_UV) return rgb(st.x - floorf(st.x), st.y - floorf(st.y), 0.0f);
    return mip_filter(sc, t, st, dx, dy);
}

// Differentials of a specular child ray (integrator.rs:164-190 reflection, 225-262 transmission).
BG_D RayDiff specular_diff(const Isect& it, const TexPoint& tp, const RayDiff& rd, V3 wi, float bsdf_eta,
                           bool transmit) {
    const SurfDiff& d = tp.d;
    RayDiff o;
    o.rxo = it.p + d.dpdx;
    o.ryo = it.p + d.dpdy;
    V3 n = it.ns;
    V3 dndx = tp.g.dndu * d.dudx + tp.g.dndv * d.dvdx;
    V3 dndy = tp.g.dndu * d.dudy + tp.g.dndv * d.dvdy;
    const V3 wo = it.wo;
    if (!transmit) {
        V3 dwodx = -rd.rxd - wo, dwody = -rd.ryd - wo;
        float ddndx = dot(dwodx, n) + dot(wo, dndx);
        float ddndy = dot(dwody, n) + dot(wo, dndy);
        o.rxd = wi - dwodx + 2.0f * (dot(wo, n) * dndx + ddndx * n);
        o.ryd = wi - dwody + 2.0f * (dot(wo, n) * dndy + ddndy * n);
        return o;
    }
    float eta = 1.0f / bsdf_eta;
    if (dot(wo, n) < 0.0f) {
        eta = 1.0f / eta;
        n = -n;
        dndx = -dndx;
        dndy = -dndy;
    }
    V3 dwodx = -rd.rxd - wo, dwody = -rd.ryd - wo;
    float ddndx = dot(dwodx, n) + dot(wo, dndx);
    float ddndy = dot(dwody, n) + dot(wo, dndy);
    float mu = eta * dot(wo, n) - abs_dot(wi, n);
    float dmudx = (eta - (eta * eta * dot(wo, n)) / abs_dot(wi, n)) * ddndx;
    float dmudy = (eta - (eta * eta * dot(wo, n)) / abs_dot(wi, n)) * ddndy;
    o.rxd = wi - eta * dwodx + (mu * dndx + dmudx * n);
    o.ryd = wi - eta * dwody + (mu * dndy + dmudy * n);
    return o;
}

}  // namespace bg

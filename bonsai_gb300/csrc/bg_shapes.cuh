// bg_shapes.cuh - triangle and sphere intersection, surface interactions, ray spawning.
//
// Device restatement of src/shapes/triangle.rs, src/shapes/sphere.rs,
// src/base/interaction.rs and src/geometries/point3.rs:31-49 with the reference's f32 operation
// order (these TUs are built with -fmad=false).  The per-ray permutation/shear constants of the
// watertight triangle test (triangle.rs:147-171) are computed once per ray instead of once per
// triangle: the values are identical, the work is not repeated.
#pragma once
#include "bg_device.h"
#include "bg_math.cuh"

namespace bg {

struct Ray {
    V3 o, d;
    float t_max;
    float time;
};

// Per-ray constants of the watertight test.
struct TriRay {
    V3 o;           // origin
    int kx, ky, kz;
    float sx, sy, sz;
};
BG_D TriRay make_tri_ray(const Ray& r) {
    TriRay t;
    t.o = r.o;
    t.kz = max_dimension(vabs(r.d));
    t.kx = t.kz + 1;
    if (t.kx == 3) t.kx = 0;
    t.ky = t.kx + 1;
    if (t.ky == 3) t.ky = 0;
    V3 d = permute(r.d, t.kx, t.ky, t.kz);
    t.sx = -d.x / d.z;
    t.sy = -d.y / d.z;
    t.sz = 1.0f / d.z;
    return t;
}

struct TriHit {
    float t, b0, b1, b2;
};

// Triangle::intersect_test / the t part of Triangle::intersect (triangle.rs:135-268).  Every
// product and sum is written with an explicitly rounded intrinsic, so the test rounds as the
// reference's f32 code in every translation unit, whatever its -fmad setting: the edge functions
// must never be contracted into fused multiply-adds, or two triangles sharing an edge could both
// reject a ray through that edge (the test would no longer be watertight).
BG_D bool tri_test(const TriRay& tr, float t_max, V3 p0, V3 p1, V3 p2, TriHit* out) {
    auto mul = [](float a, float b) { return __fmul_rn(a, b); };
    auto add = [](float a, float b) { return __fadd_rn(a, b); };
    auto sub = [](float a, float b) { return __fsub_rn(a, b); };
    V3 p0t = permute(v3(sub(p0.x, tr.o.x), sub(p0.y, tr.o.y), sub(p0.z, tr.o.z)), tr.kx, tr.ky, tr.kz);
    V3 p1t = permute(v3(sub(p1.x, tr.o.x), sub(p1.y, tr.o.y), sub(p1.z, tr.o.z)), tr.kx, tr.ky, tr.kz);
    V3 p2t = permute(v3(sub(p2.x, tr.o.x), sub(p2.y, tr.o.y), sub(p2.z, tr.o.z)), tr.kx, tr.ky, tr.kz);
    p0t.x = add(p0t.x, mul(tr.sx, p0t.z));
    p0t.y = add(p0t.y, mul(tr.sy, p0t.z));
    p1t.x = add(p1t.x, mul(tr.sx, p1t.z));
    p1t.y = add(p1t.y, mul(tr.sy, p1t.z));
    p2t.x = add(p2t.x, mul(tr.sx, p2t.z));
    p2t.y = add(p2t.y, mul(tr.sy, p2t.z));
    float e0 = sub(mul(p1t.x, p2t.y), mul(p1t.y, p2t.x));
    float e1 = sub(mul(p2t.x, p0t.y), mul(p2t.y, p0t.x));
    float e2 = sub(mul(p0t.x, p1t.y), mul(p0t.y, p1t.x));
    if (e0 == 0.0f || e1 == 0.0f || e2 == 0.0f) {  // triangle.rs:178-190 (f64 there)
        e0 = diff_of_products(p1t.x, p2t.y, p1t.y, p2t.x);
        e1 = diff_of_products(p2t.x, p0t.y, p2t.y, p0t.x);
        e2 = diff_of_products(p0t.x, p1t.y, p0t.y, p1t.x);
    }
    if ((e0 < 0.0f || e1 < 0.0f || e2 < 0.0f) && (e0 > 0.0f || e1 > 0.0f || e2 > 0.0f)) return false;
    float det = add(add(e0, e1), e2);
    if (det == 0.0f) return false;
    p0t.z = mul(p0t.z, tr.sz);
    p1t.z = mul(p1t.z, tr.sz);
    p2t.z = mul(p2t.z, tr.sz);
    float ts = add(add(mul(e0, p0t.z), mul(e1, p1t.z)), mul(e2, p2t.z));
    if (det < 0.0f && (ts >= 0.0f || ts < mul(t_max, det))) return false;
    else if (det > 0.0f && (ts <= 0.0f || ts > mul(t_max, det))) return false;
    float inv_det = 1.0f / det;
    float t = mul(ts, inv_det);
    // conservative t bound (triangle.rs:219-239)
    float max_zt = max_component(vabs(v3(p0t.z, p1t.z, p2t.z)));
    float delta_z = mul(gamma(3.0f), max_zt);
    float max_xt = max_component(vabs(v3(p0t.x, p1t.x, p2t.x)));
    float max_yt = max_component(vabs(v3(p0t.y, p1t.y, p2t.y)));
    float delta_x = mul(gamma(5.0f), add(max_xt, max_zt));
    float delta_y = mul(gamma(5.0f), add(max_yt, max_zt));
    float delta_e = mul(2.0f, add(add(mul(mul(gamma(2.0f), max_xt), max_yt), mul(delta_y, max_xt)), mul(delta_x, max_yt)));
    float max_e = max_component(vabs(v3(e0, e1, e2)));
    float delta_t = mul(mul(3.0f, add(add(mul(mul(gamma(3.0f), max_e), max_zt), mul(delta_e, max_zt)), mul(delta_z, max_e))),
                        fabsf(inv_det));
    if (t <= delta_t) return false;
    // degenerate-triangle exit (triangle.rs:241-268 with the default uvs): rejected only when both
    // dpdu x dpdv and (p2-p0)x(p1-p0) vanish
    V3 ng = cross(p2 - p0, p1 - p0);
    if (length_squared(ng) == 0.0f) {
        V3 dp02 = p0 - p2, dp12 = p1 - p2;
        V3 dpdu = (-1.0f * dp02 - -1.0f * dp12) * 1.0f;
        V3 dpdv = (-0.0f * dp02 + -1.0f * dp12) * 1.0f;
        if (length_squared(cross(dpdu, dpdv)) == 0.0f) return false;
    }
    if (out) {
        out->t = t;
        out->b0 = mul(e0, inv_det);
        out->b1 = mul(e1, inv_det);
        out->b2 = mul(e2, inv_det);
    }
    return true;
}

// Surface interaction (geometry part of SurfaceInteraction) used by shading.
struct Isect {
    V3 p, p_err, wo, n, ns, dpdu;  // dpdu = shading dpdu (BSDF s axis before normalisation)
    float time;
    int prim;
};

// The parts of a SurfaceInteraction that only textures and ray differentials read: the (u,v)
// parameterisation, the geometric partials dpdu / dpdv and the shading normal's partials
// (interaction.rs:18-55).  Computed on demand (prim_geom) so plain shading does not carry them.
struct SurfaceGeom {
    float u, v;
    V3 dpdu, dpdv;  // geometric (SurfaceInteraction::dpdu / dpdv)
    V3 dndu, dndv;  // shading (Shading::dndu / dndv)
};

// Vec3::coordinate_system (vec3.rs:25-33)
BG_D void coordinate_system(V3 v1, V3* v2, V3* v3o) {
    if (fabsf(v1.x) > fabsf(v1.y)) *v2 = v3(-v1.z, 0.0f, v1.x) / sqrtf(v1.x * v1.x + v1.z * v1.z);
    else *v2 = v3(0.0f, v1.z, -v1.y) / sqrtf(v1.y * v1.y + v1.z * v1.z);
    *v3o = cross(v1, *v2);
}

// Triangle interaction without vertex attributes (default uvs (0,0),(1,0),(1,1), no shading
// normals, no orientation flip): triangle.rs:241-307 with the uv deltas folded.
BG_D void tri_isect_plain(V3 p0, V3 p1, V3 p2, const TriHit& h, const Ray& ray, Isect* it) {
    V3 dp02 = p0 - p2, dp12 = p1 - p2;
    // default uvs (0,0),(1,0),(1,1): duv02=(-1,-1), duv12=(0,-1), determinant 1
    V3 dpdu = (-1.0f * dp02 - -1.0f * dp12) * 1.0f;
    V3 dpdv = (-0.0f * dp02 + -1.0f * dp12) * 1.0f;
    if (length_squared(cross(dpdu, dpdv)) == 0.0f) {
        V3 ng = normalize(cross(p2 - p0, p1 - p0));
        coordinate_system(ng, &dpdu, &dpdv);
    }
    float xs = fabsf(h.b0 * p0.x) + fabsf(h.b1 * p1.x) + fabsf(h.b2 * p2.x);
    float ys = fabsf(h.b0 * p0.y) + fabsf(h.b1 * p1.y) + fabsf(h.b2 * p2.y);
    float zs = fabsf(h.b0 * p0.z) + fabsf(h.b1 * p1.z) + fabsf(h.b2 * p2.z);
    it->p_err = gamma(7.0f) * v3(xs, ys, zs);
    it->p = h.b0 * p0 + h.b1 * p1 + h.b2 * p2;
    it->time = ray.time;
    it->wo = -ray.d;
    V3 nn = normalize(cross(dp02, dp12));
    it->n = nn;
    it->ns = nn;
    it->dpdu = dpdu;
}

BG_D uint8_t tri_flag_bits(const Scene& sc, uint32_t prim) { return sc.tri_flags ? sc.tri_flags[prim] : (uint8_t)0; }
// Triangle::get_uvs (triangle.rs:107-117)
BG_D void tri_uvs(const Scene& sc, uint32_t prim, float2 uv[3]) {
    if (sc.tri_uv) {
        uv[0] = sc.tri_uv[3 * prim];
        uv[1] = sc.tri_uv[3 * prim + 1];
        uv[2] = sc.tri_uv[3 * prim + 2];
    } else {
        uv[0] = make_float2(0.0f, 0.0f);
        uv[1] = make_float2(1.0f, 0.0f);
        uv[2] = make_float2(1.0f, 1.0f);
    }
}

// Triangle::intersect's interaction with the mesh's vertex attributes (triangle.rs:241-400):
// partials from the vertex uvs, the geometric normal flipped for reverse_orientation ^
// transform_swaps_handedness, and with vertex normals the shading frame of
// Interaction::set_shading_geometry (interaction.rs:145-168, orientation authoritative).
BG_D void tri_isect(const Scene& sc, uint32_t prim, V3 p0, V3 p1, V3 p2, const TriHit& h, const Ray& ray, Isect* it,
                    SurfaceGeom* g = nullptr) {
    const uint8_t fl = tri_flag_bits(sc, prim);
    if (!sc.tri_uv && fl == 0 && !g) {
        tri_isect_plain(p0, p1, p2, h, ray, it);
        return;
    }
    float2 uv[3];
    tri_uvs(sc, prim, uv);
    const float du02 = uv[0].x - uv[2].x, dv02 = uv[0].y - uv[2].y;
    const float du12 = uv[1].x - uv[2].x, dv12 = uv[1].y - uv[2].y;
    V3 dp02 = p0 - p2, dp12 = p1 - p2;
    const float det = du02 * dv12 - dv02 * du12;
    const bool degenerate_uv = fabsf(det) < 1e-8f;
    V3 dpdu = v3(0.0f, 0.0f, 0.0f), dpdv = v3(0.0f, 0.0f, 0.0f);
    if (!degenerate_uv) {
        float inv = 1.0f / det;
        dpdu = (dv12 * dp02 - dv02 * dp12) * inv;
        dpdv = (-du12 * dp02 + du02 * dp12) * inv;
    }
    if (degenerate_uv || length_squared(cross(dpdu, dpdv)) == 0.0f) {
        V3 ng = cross(p2 - p0, p1 - p0);
        coordinate_system(normalize(ng), &dpdu, &dpdv);
    }
    float xs = fabsf(h.b0 * p0.x) + fabsf(h.b1 * p1.x) + fabsf(h.b2 * p2.x);
    float ys = fabsf(h.b0 * p0.y) + fabsf(h.b1 * p1.y) + fabsf(h.b2 * p2.y);
    float zs = fabsf(h.b0 * p0.z) + fabsf(h.b1 * p1.z) + fabsf(h.b2 * p2.z);
    it->p_err = gamma(7.0f) * v3(xs, ys, zs);
    it->p = h.b0 * p0 + h.b1 * p1 + h.b2 * p2;
    it->time = ray.time;
    it->wo = -ray.d;
    V3 nn = normalize(cross(dp02, dp12));
    if (((fl & TRI_REVERSE) != 0) != ((fl & TRI_SWAPS) != 0)) nn = -nn;
    it->n = nn;
    it->ns = nn;
    it->dpdu = dpdu;
    V3 dndu = v3(0.0f, 0.0f, 0.0f), dndv = v3(0.0f, 0.0f, 0.0f);
    if (fl & TRI_NORMALS) {
        const V3 n0 = f4xyz(sc.tri_ns[3 * prim]), n1 = f4xyz(sc.tri_ns[3 * prim + 1]),
                 n2 = f4xyz(sc.tri_ns[3 * prim + 2]);
        V3 sn = h.b0 * n0 + h.b1 * n1 + h.b2 * n2;
        sn = length_squared(sn) > 0.0f ? normalize(sn) : it->n;
        V3 st = normalize(dpdu);
        V3 sb = cross(st, sn);
        if (length_squared(sb) > 0.0f) {
            sb = normalize(sb);
            st = cross(sb, sn);
        } else {
            coordinate_system(sn, &st, &sb);
        }
        if (g) {
            V3 dn1 = n0 - n2, dn2 = n1 - n2;
            if (degenerate_uv) {
                V3 dn = cross(n2 - n0, n1 - n0);
                if (length_squared(dn) != 0.0f) coordinate_system(dn, &dndu, &dndv);
            } else {
                float inv = 1.0f / det;
                dndu = (dv12 * dn1 - dv02 * dn2) * inv;
                dndv = (-du12 * dn1 + du02 * dn2) * inv;
            }
        }
        if (fl & TRI_REVERSE) sb = -sb;
        V3 ns = normalize(cross(st, sb));
        it->n = face_forward(it->n, ns);
        it->ns = ns;
        it->dpdu = st;
    }
    if (g) {
        g->u = (h.b0 * uv[0].x + h.b1 * uv[1].x) + h.b2 * uv[2].x;
        g->v = (h.b0 * uv[0].y + h.b1 * uv[1].y) + h.b2 * uv[2].y;
        g->dpdu = dpdu;
        g->dpdv = dpdv;
        g->dndu = dndu;
        g->dndv = dndv;
    }
}

BG_D float tri_area(V3 p0, V3 p1, V3 p2) { return 0.5f * length(cross(p1 - p0, p2 - p0)); }

// Sphere with object_to_world = translate(c): world_to_object is translate(-c) (translate(0)
// itself when c == 0, sphere.rs:40-45).  xo = (1*x + 0*y) + (0*z + m03), as point3.rs:71-100.
struct SphereXf {
    V3 c;       // center (object_to_world translation)
    V3 ci;      // world_to_object translation
};
BG_D SphereXf sphere_xf(float4 s) {
    SphereXf x;
    x.c = v3(s.x, s.y, s.z);
    bool ident = (s.x == 0.0f && s.y == 0.0f && s.z == 0.0f);
    x.ci = ident ? x.c : v3(-s.x, -s.y, -s.z);
    return x;
}
BG_D V3 xf_point_err(V3 t, V3 p, V3* err) {  // rows (1,0,0,tx) (0,1,0,ty) (0,0,1,tz)
    float xp = (1.0f * p.x + 0.0f * p.y) + (0.0f * p.z + t.x);
    float yp = (0.0f * p.x + 1.0f * p.y) + (0.0f * p.z + t.y);
    float zp = (0.0f * p.x + 0.0f * p.y) + (1.0f * p.z + t.z);
    float xa = fabsf(1.0f * p.x) + fabsf(0.0f * p.y) + fabsf(0.0f * p.z) + fabsf(t.x);
    float ya = fabsf(0.0f * p.x) + fabsf(1.0f * p.y) + fabsf(0.0f * p.z) + fabsf(t.y);
    float za = fabsf(0.0f * p.x) + fabsf(0.0f * p.y) + fabsf(1.0f * p.z) + fabsf(t.z);
    *err = gamma(3.0f) * v3(xa, ya, za);
    return v3(xp, yp, zp);
}
BG_D V3 xf_vec_id(V3 v) {  // identity 3x3 rows
    return v3(1.0f * v.x + 0.0f * v.y + 0.0f * v.z, 0.0f * v.x + 1.0f * v.y + 0.0f * v.z,
              0.0f * v.x + 0.0f * v.y + 1.0f * v.z);
}
BG_D V3 xf_vec_err_id(V3 v, V3* e) {
    float g3 = gamma(3.0f);
    e->x = g3 * (fabsf(1.0f * v.x) + fabsf(0.0f * v.y) + fabsf(0.0f * v.z));
    e->y = g3 * (fabsf(0.0f * v.x) + fabsf(1.0f * v.y) + fabsf(0.0f * v.z));
    e->z = g3 * (fabsf(0.0f * v.x) + fabsf(0.0f * v.y) + fabsf(1.0f * v.z));
    return xf_vec_id(v);
}

// Normal partials from the fundamental forms (sphere.rs:191-204, cylinder.rs:161-179,
// cone.rs:161-179).
BG_D void weingarten(V3 dpdu, V3 dpdv, V3 d2pduu, V3 d2pduv, V3 d2pdvv, V3* dndu, V3* dndv) {
    float e1 = dot(dpdu, dpdu), f1 = dot(dpdu, dpdv), g1 = dot(dpdv, dpdv);
    V3 n = normalize(cross(dpdu, dpdv));
    float e2 = dot(n, d2pduu), f2 = dot(n, d2pduv), g2 = dot(n, d2pdvv);
    float inv_egf = 1.0f / (e1 * g1 - f1 * f1);
    *dndu = (f2 * f1 - e2 * g1) * inv_egf * dpdu + (e2 * f1 - f2 * e1) * inv_egf * dpdv;
    *dndv = (g2 * f1 - f2 * g1) * inv_egf * dpdu + (f2 * f1 - g2 * e1) * inv_egf * dpdv;
}

struct SphHit {
    float t;
    Ray ray_obj;  // object-space ray with the origin moved to the error bound (ray.rs:78-106)
};

// Sphere::intersect / intersect_test for a full sphere (sphere.rs:80-161, 239-326).
BG_D bool sphere_test(float4 s, const Ray& rw, float t_max, SphHit* out) {
    SphereXf xf = sphere_xf(s);
    float radius = s.w;
    V3 oe, de;
    Ray ray;
    ray.o = xf_point_err(xf.ci, rw.o, &oe);
    ray.d = xf_vec_err_id(rw.d, &de);
    ray.t_max = t_max;
    ray.time = rw.time;
    float ls = length_squared(ray.d);
    if (ls > 0.0f) {
        float dt = dot(vabs(ray.d), oe) / ls;
        ray.o = ray.o + ray.d * dt;
    }
    EF ox = ef(ray.o.x, oe.x), oy = ef(ray.o.y, oe.y), oz = ef(ray.o.z, oe.z);
    EF dx = ef(ray.d.x, de.x), dy = ef(ray.d.y, de.y), dz = ef(ray.d.z, de.z);
    EF a = dx * dx + dy * dy + dz * dz;
    EF b = ef(2.0f) * (dx * ox + dy * oy + dz * oz);
    EF c = ox * ox + oy * oy + oz * oz - ef(radius) * ef(radius);
    EF t0, t1;
    if (!quadratic(a, b, c, &t0, &t1)) return false;
    if (t0.hi > t_max || t1.lo <= 0.0f) return false;
    EF tsh = t0;
    if (tsh.lo <= 0.0f) {
        tsh = t1;
        if (tsh.hi > t_max) return false;
    }
    // full sphere: the z-range / phi_max clipping of sphere.rs:127-161 never triggers
    if (out) {
        out->t = tsh.v;
        out->ray_obj = ray;
    }
    return true;
}

// Sphere interaction (sphere.rs:163-236 + Interaction::transform, interaction.rs:268-300).
BG_D void sphere_isect(float4 s, const SphHit& h, const Ray& rw, Isect* it, SurfaceGeom* g = nullptr) {
    const float radius = s.w;
    const float phi_max = 360.0f * (PI / 180.0f);
    const float theta_min = acosf(rclamp(-radius / radius, -1.0f, 1.0f));
    const float theta_max = acosf(rclamp(radius / radius, -1.0f, 1.0f));
    V3 ph = h.ray_obj.o + h.ray_obj.d * h.t;  // refine (sphere.rs:119-124)
    ph = ph * (radius / length(ph - v3(0.0f, 0.0f, 0.0f)));
    if (ph.x == 0.0f && ph.y == 0.0f) ph.x = 1e-5f * radius;
    float theta = acosf(rclamp(ph.z / radius, -1.0f, 1.0f));
    float z_radius = sqrtf(ph.x * ph.x + ph.y * ph.y);
    float inv_zr = 1.0f / z_radius;
    float cos_phi = ph.x * inv_zr, sin_phi = ph.y * inv_zr;
    V3 dpdu = v3(-phi_max * ph.y, phi_max * ph.x, 0.0f);
    V3 dpdv = (theta_max - theta_min) * v3(ph.z * cos_phi, ph.z * sin_phi, -radius * sinf(theta));
    V3 perr = gamma(5.0f) * vabs(ph);
    V3 n = normalize(cross(dpdu, dpdv));
    SphereXf xf = sphere_xf(s);
    // transform_with_point_error (point3.rs:102-140) with translation xf.c
    float g3 = gamma(3.0f);
    V3 p;
    p.x = (1.0f * ph.x + 0.0f * ph.y) + (0.0f * ph.z + xf.c.x);
    p.y = (0.0f * ph.x + 1.0f * ph.y) + (0.0f * ph.z + xf.c.y);
    p.z = (0.0f * ph.x + 0.0f * ph.y) + (1.0f * ph.z + xf.c.z);
    V3 ae;
    ae.x = (g3 + 1.0f) * (1.0f * perr.x + 0.0f * perr.y + 0.0f * perr.z) +
           g3 * (fabsf(1.0f * ph.x) + fabsf(0.0f * ph.y) + fabsf(0.0f * ph.z) + fabsf(xf.c.x));
    ae.y = (g3 + 1.0f) * (0.0f * perr.x + 1.0f * perr.y + 0.0f * perr.z) +
           g3 * (fabsf(0.0f * ph.x) + fabsf(1.0f * ph.y) + fabsf(0.0f * ph.z) + fabsf(xf.c.y));
    ae.z = (g3 + 1.0f) * (0.0f * perr.x + 0.0f * perr.y + 1.0f * perr.z) +
           g3 * (fabsf(0.0f * ph.x) + fabsf(0.0f * ph.y) + fabsf(1.0f * ph.z) + fabsf(xf.c.z));
    it->p = p;
    it->p_err = ae;
    it->time = rw.time;
    it->wo = xf_vec_id(-h.ray_obj.d);
    // Normal::transform uses m_inverse^T: identity 3x3 for a translation
    V3 nt = xf_vec_id(n);
    it->n = normalize(nt);
    it->ns = face_forward(normalize(nt), it->n);
    it->dpdu = xf_vec_id(dpdu);
    if (g) {  // sphere.rs:165-204: (u, v) and the Weingarten normal derivatives
        float phi = atan2f(ph.y, ph.x);
        if (phi < 0.0f) phi += 2.0f * PI;
        g->u = phi / phi_max;
        g->v = (theta - theta_min) / (theta_max - theta_min);
        V3 d2pduu = -phi_max * phi_max * v3(ph.x, ph.y, 0.0f);
        V3 d2pduv = (theta_max - theta_min) * ph.z * phi_max * v3(-sin_phi, cos_phi, 0.0f);
        V3 d2pdvv = -(theta_max - theta_min) * (theta_max - theta_min) * ph;
        weingarten(dpdu, dpdv, d2pduu, d2pduv, d2pdvv, &g->dndu, &g->dndv);
        g->dpdu = xf_vec_id(dpdu);
        g->dpdv = xf_vec_id(dpdv);
        g->dndu = xf_vec_id(g->dndu);  // Normal::transform with the identity m_inverse
        g->dndv = xf_vec_id(g->dndv);
    }
}

// ---------------------------------------------------------------- quadrics (cylinder, disk, cone)
struct M34 {
    float m[3][4];
};
BG_D M34 load_m34(const float4* r) {
    M34 x;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float4 v = r[i];
        x.m[i][0] = v.x;
        x.m[i][1] = v.y;
        x.m[i][2] = v.z;
        x.m[i][3] = v.w;
    }
    return x;
}
// Point3::transform_with_error / Vec3::transform(_with_error) / Normal::transform with a 3x4 affine
// matrix (bottom row 0 0 0 1, so the homogeneous w is exactly 1) - point3.rs:71-140, vec3.rs:35-64.
BG_D V3 m_point_err(const M34& t, V3 p, V3* err) {
    const auto& m = t.m;
    float xp = (m[0][0] * p.x + m[0][1] * p.y) + (m[0][2] * p.z + m[0][3]);
    float yp = (m[1][0] * p.x + m[1][1] * p.y) + (m[1][2] * p.z + m[1][3]);
    float zp = (m[2][0] * p.x + m[2][1] * p.y) + (m[2][2] * p.z + m[2][3]);
    float xa = fabsf(m[0][0] * p.x) + fabsf(m[0][1] * p.y) + fabsf(m[0][2] * p.z) + fabsf(m[0][3]);
    float ya = fabsf(m[1][0] * p.x) + fabsf(m[1][1] * p.y) + fabsf(m[1][2] * p.z) + fabsf(m[1][3]);
    float za = fabsf(m[2][0] * p.x) + fabsf(m[2][1] * p.y) + fabsf(m[2][2] * p.z) + fabsf(m[2][3]);
    *err = gamma(3.0f) * v3(xa, ya, za);
    return v3(xp, yp, zp);
}
BG_D V3 m_vec(const M34& t, V3 v) {
    const auto& m = t.m;
    return v3(m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z, m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z,
              m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z);
}
BG_D V3 m_vec_err(const M34& t, V3 v, V3* e) {
    const auto& m = t.m;
    float g3 = gamma(3.0f);
    e->x = g3 * (fabsf(m[0][0] * v.x) + fabsf(m[0][1] * v.y) + fabsf(m[0][2] * v.z));
    e->y = g3 * (fabsf(m[1][0] * v.x) + fabsf(m[1][1] * v.y) + fabsf(m[1][2] * v.z));
    e->z = g3 * (fabsf(m[2][0] * v.x) + fabsf(m[2][1] * v.y) + fabsf(m[2][2] * v.z));
    return m_vec(t, v);
}
BG_D V3 m_normal(const M34& inv, V3 n) {  // uses m_inverse transposed
    const auto& mi = inv.m;
    return v3(mi[0][0] * n.x + mi[1][0] * n.y + mi[2][0] * n.z, mi[0][1] * n.x + mi[1][1] * n.y + mi[2][1] * n.z,
              mi[0][2] * n.x + mi[1][2] * n.y + mi[2][2] * n.z);
}
BG_D V3 m_point_perr(const M34& t, V3 p, V3 pe, V3* ae) {
    const auto& m = t.m;
    float g3 = gamma(3.0f);
    V3 r;
    r.x = (m[0][0] * p.x + m[0][1] * p.y) + (m[0][2] * p.z + m[0][3]);
    r.y = (m[1][0] * p.x + m[1][1] * p.y) + (m[1][2] * p.z + m[1][3]);
    r.z = (m[2][0] * p.x + m[2][1] * p.y) + (m[2][2] * p.z + m[2][3]);
    ae->x = (g3 + 1.0f) * (fabsf(m[0][0]) * pe.x + fabsf(m[0][1]) * pe.y + fabsf(m[0][2]) * pe.z) +
            g3 * (fabsf(m[0][0] * p.x) + fabsf(m[0][1] * p.y) + fabsf(m[0][2] * p.z) + fabsf(m[0][3]));
    ae->y = (g3 + 1.0f) * (fabsf(m[1][0]) * pe.x + fabsf(m[1][1]) * pe.y + fabsf(m[1][2]) * pe.z) +
            g3 * (fabsf(m[1][0] * p.x) + fabsf(m[1][1] * p.y) + fabsf(m[1][2] * p.z) + fabsf(m[1][3]));
    ae->z = (g3 + 1.0f) * (fabsf(m[2][0]) * pe.x + fabsf(m[2][1]) * pe.y + fabsf(m[2][2]) * pe.z) +
            g3 * (fabsf(m[2][0] * p.x) + fabsf(m[2][1] * p.y) + fabsf(m[2][2] * p.z) + fabsf(m[2][3]));
    return r;
}
BG_D float ef_abs_err(EF e) { return next_float_up(rmax(fabsf(e.hi - e.v), fabsf(e.v - e.lo))); }

// Cylinder / Disk / Cone ::intersect and ::intersect_test (cylinder.rs:71-288, disk.rs:70-183,
// cone.rs:67-287).  Fills `it` (world-space interaction) when it is non-null.
BG_D bool quadric_hit(const float4* q, const Ray& rw, float t_max, float* t_out, Isect* it,
                      SurfaceGeom* g = nullptr) {
    const float4 p0 = q[6], p1 = q[7];
    const uint32_t flags = __float_as_uint(p1.z);
    const int kind = (int)(flags & 0xFFu);
    const float radius = p0.x, inner = p0.y, z_min = p0.z, z_max = p0.w, height = p1.x, phi_max = p1.y;
    const M34 w2o = load_m34(q + 3);
    V3 oe, de;
    Ray ray;
    ray.o = m_point_err(w2o, rw.o, &oe);
    ray.d = m_vec_err(w2o, rw.d, &de);
    ray.t_max = t_max;
    ray.time = rw.time;
    float ls = length_squared(ray.d);
    if (ls > 0.0f) {
        float dt = dot(vabs(ray.d), oe) / ls;
        ray.o = ray.o + ray.d * dt;
    }
    V3 ph, dpdu, dpdv, perr;
    V3 d2pduu = v3(0.0f, 0.0f, 0.0f), d2pduv = v3(0.0f, 0.0f, 0.0f);
    float tsh_v, gu = 0.0f, gv = 0.0f;
    if (kind == 1) {  // disk
        if (ray.d.z == 0.0f) return false;
        float tsh = (height - ray.o.z) / ray.d.z;
        if (tsh <= 0.0f || tsh >= ray.t_max) return false;
        ph = ray.o + ray.d * tsh;
        float dist = ph.x * ph.x + ph.y * ph.y;
        if (dist > radius * radius || dist < inner * inner) return false;
        float phi = atan2f(ph.y, ph.x);
        if (phi < 0.0f) phi += 2.0f * PI;
        if (phi > phi_max) return false;
        if (!it) {
            *t_out = tsh;
            return true;
        }
        float rh = sqrtf(dist);
        gu = phi / phi_max;  // disk.rs:106-113 (dndu = dndv = 0)
        gv = (radius - rh) / (radius - inner);
        dpdu = v3(-phi_max * ph.y, phi_max * ph.x, 0.0f);
        dpdv = v3(ph.x, ph.y, 0.0f) * (inner - radius) / rh;
        ph.z = height;
        perr = v3(0.0f, 0.0f, 0.0f);
        tsh_v = tsh;
    } else {
        EF ox = ef(ray.o.x, oe.x), oy = ef(ray.o.y, oe.y), oz = ef(ray.o.z, oe.z);
        EF dx = ef(ray.d.x, de.x), dy = ef(ray.d.y, de.y), dz = ef(ray.d.z, de.z);
        EF a, b, c;
        if (kind == 0) {
            a = dx * dx + dy * dy;
            b = ef(2.0f) * (dx * ox + dy * oy);
            c = ox * ox + oy * oy - ef(radius, 0.0f) * ef(radius, 0.0f);
        } else {
            EF k = ef(radius, 0.0f) / ef(height, 0.0f);
            k = k * k;
            a = dx * dx + dy * dy - k * dz * dz;
            b = ef(2.0f) * (dx * ox + dy * oy - k * dz * (oz - ef(height)));
            c = ox * ox + oy * oy - k * (oz - ef(height)) * (oz - ef(height));
        }
        EF t0, t1;
        if (!quadratic(a, b, c, &t0, &t1)) return false;
        if (t0.hi > ray.t_max || t1.lo <= 0.0f) return false;
        EF tsh = t0;
        if (tsh.lo <= 0.0f) {
            tsh = t1;
            if (tsh.hi > ray.t_max) return false;
        }
        bool used_t1 = tsh.v == t1.v && tsh.lo == t1.lo && tsh.hi == t1.hi;
        float phi = 0.0f;
        for (int pass = 0; pass < 2; ++pass) {
            ph = ray.o + ray.d * tsh.v;
            if (kind == 0) {
                float hr = sqrtf(ph.x * ph.x + ph.y * ph.y);
                ph.x *= radius / hr;
                ph.y *= radius / hr;
            }
            phi = atan2f(ph.y, ph.x);
            if (phi < 0.0f) phi += 2.0f * PI;
            bool clipped = kind == 0 ? (ph.z < z_min || ph.z > z_max || phi > phi_max)
                                     : (ph.z < 0.0f || ph.z > height || phi > phi_max);
            if (!clipped) break;
            if (pass == 1 || used_t1) return false;
            if (t1.hi > ray.t_max) return false;
            tsh = t1;
            used_t1 = true;
        }
        if (!it) {
            *t_out = tsh.v;
            return true;
        }
        dpdu = v3(-phi_max * ph.y, phi_max * ph.x, 0.0f);
        gu = phi / phi_max;
        d2pduu = -phi_max * phi_max * v3(ph.x, ph.y, 0.0f);
        if (kind == 0) {
            gv = (ph.z - z_min) / (z_max - z_min);
            dpdv = v3(0.0f, 0.0f, z_max - z_min);
            perr = gamma(3.0f) * vabs(v3(ph.x, ph.y, 0.0f));
        } else {
            float v = ph.z / height;
            gv = v;
            dpdv = v3(-ph.x / (1.0f - v), -ph.y / (1.0f - v), height);
            d2pduv = phi_max / (1.0f - v) * v3(ph.y, -ph.x, 0.0f);
            EF px = ox + tsh * dx, py = oy + tsh * dy, pz = oz + tsh * dz;
            perr = v3(ef_abs_err(px), ef_abs_err(py), ef_abs_err(pz));
        }
        tsh_v = tsh.v;
    }
    // Interaction::new + Interaction::transform(object_to_world)
    const M34 o2w = load_m34(q);
    V3 n = normalize(cross(dpdu, dpdv));
    if (((flags >> 8) & 1u) ^ ((flags >> 9) & 1u)) n = n * -1.0f;
    V3 ae;
    it->p = m_point_perr(o2w, ph, perr, &ae);
    it->p_err = ae;
    it->time = ray.time;
    it->wo = m_vec(o2w, -ray.d);
    it->n = normalize(m_normal(w2o, n));
    it->ns = face_forward(normalize(m_normal(w2o, n)), it->n);
    it->dpdu = m_vec(o2w, dpdu);
    if (g) {
        V3 dndu = v3(0.0f, 0.0f, 0.0f), dndv = v3(0.0f, 0.0f, 0.0f);
        if (kind != 1) weingarten(dpdu, dpdv, d2pduu, d2pduv, v3(0.0f, 0.0f, 0.0f), &dndu, &dndv);
        g->u = gu;
        g->v = gv;
        g->dpdu = m_vec(o2w, dpdu);
        g->dpdv = m_vec(o2w, dpdv);
        g->dndu = m_normal(w2o, dndu);
        g->dndv = m_normal(w2o, dndv);
    }
    *t_out = tsh_v;
    return true;
}

// Point3::offset_ray_origin (point3.rs:31-49)
BG_D V3 offset_ray_origin(V3 p, V3 perr, V3 n, V3 w) {
    V3 offset = dot(vabs(n), perr) * n;
    if (dot(w, n) < 0.0f) offset = -offset;
    V3 po = p + offset;
    if (offset.x > 0.0f) po.x = next_float_up(po.x);
    else if (offset.x < 0.0f) po.x = next_float_down(po.x);
    if (offset.y > 0.0f) po.y = next_float_up(po.y);
    else if (offset.y < 0.0f) po.y = next_float_down(po.y);
    if (offset.z > 0.0f) po.z = next_float_up(po.z);
    else if (offset.z < 0.0f) po.z = next_float_down(po.z);
    return po;
}
// Interaction::spawn_ray (interaction.rs:115-121): t_max 1 - 0.0001 in the reference (F3),
// infinity in PBRT mode.
BG_D Ray spawn_ray(V3 p, V3 perr, V3 n, float time, V3 d, bool ref_compat) {
    Ray r;
    r.o = offset_ray_origin(p, perr, n, d);
    r.d = d;
    r.t_max = ref_compat ? (1.0f - 0.0001f) : INFINITY;
    r.time = time;
    return r;
}
// Interaction::spawn_ray_to_it (interaction.rs:132-143)
BG_D Ray spawn_ray_to(V3 p, V3 perr, V3 n, float time, V3 q, V3 qerr, V3 qn) {
    V3 o = offset_ray_origin(p, perr, n, q - p);
    V3 target = offset_ray_origin(q, qerr, qn, o - q);
    Ray r;
    r.o = o;
    r.d = target - o;
    r.t_max = 1.0f - 0.0001f;
    r.time = time;
    return r;
}

// Triangle::sample (triangle.rs:522-559) with uniform_sample_triangle (sampling.rs:233-236).
struct ShapeSample {
    V3 p, p_err, n;
    float pdf_area;
    float b0, b1;
};
BG_D ShapeSample tri_sample(V3 p0, V3 p1, V3 p2, float u0, float u1) {
    ShapeSample s;
    float sq = sqrtf(u0);
    float b0 = 1.0f - sq, b1 = u1 * sq;
    float b2 = 1.0f - b0 - b1;
    s.p = b0 * p0 + b1 * p1 + b2 * p2;
    s.n = normalize(cross(p1 - p0, p2 - p0));
    V3 pabs = vabs(b0 * p0) + vabs(b1 * p1) + vabs(b2 * p2);
    s.p_err = gamma(6.0f) * pabs;
    s.pdf_area = 1.0f / tri_area(p0, p1, p2);
    s.b0 = b0;
    s.b1 = b1;
    return s;
}

BG_D void load_tri(const Scene& sc, uint32_t prim, V3* p0, V3* p1, V3* p2) {
    float4 a = sc.tri[3 * prim], b = sc.tri[3 * prim + 1], c = sc.tri[3 * prim + 2];
    *p0 = f4xyz(a);
    *p1 = f4xyz(b);
    *p2 = f4xyz(c);
}

// Full closest-hit interaction for a primitive given the ray (re-runs the shape test with
// t_max = infinity, which reproduces the traversal's t, barycentrics and hit side).
// With `g`, also the surface parameterisation and partials (SurfaceGeom).
BG_D bool prim_isect(const Scene& sc, int prim, const Ray& ray, Isect* it, SurfaceGeom* g = nullptr) {
    if ((uint32_t)prim < sc.ntri) {
        V3 p0, p1, p2;
        load_tri(sc, (uint32_t)prim, &p0, &p1, &p2);
        TriRay tr = make_tri_ray(ray);
        TriHit h;
        if (!tri_test(tr, INFINITY, p0, p1, p2, &h)) return false;
        tri_isect(sc, (uint32_t)prim, p0, p1, p2, h, ray, it, g);
    } else if ((uint32_t)prim < sc.ntri + sc.nsph) {
        float4 s = sc.sph[prim - sc.ntri];
        SphHit h;
        if (!sphere_test(s, ray, INFINITY, &h)) return false;
        sphere_isect(s, h, ray, it, g);
    } else {
        float t;
        if (!quadric_hit(sc.quads + QUADRIC_F4 * (prim - sc.ntri - sc.nsph), ray, INFINITY, &t, it, g)) return false;
    }
    it->prim = prim;
    return true;
}

}  // namespace bg

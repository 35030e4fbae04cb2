// bg_shading.cuh - BxDFs, BSDF, materials, area lights and the perspective camera on the device.
//
// Restates src/base/{bsdf,bxdf,microfacet,fresnel}.rs, src/bxdfs/{lambertian,microfacet,fresnel}.rs,
// src/materials/{matte,plastic}.rs, src/lights/diffuse.rs, src/base/shape.rs:17-57,
// src/base/sampling.rs and src/cameras/perspective.rs.  REF selects the reference's own
// behaviour where it deviates from PBRT-v3 (F4 G1 = lambda, F5 slope_x_1, F8 component counter,
// F12 emission toward +wi, F13 light pdf without 1/area, F14 Fresnel without |cos|).
#pragma once
#include "bg_device.h"
#include "bg_math.cuh"
#include "bg_shapes.cuh"
#include "bg_texture.cuh"

namespace bg {

enum : uint8_t {
    BSDF_REFLECTION = 1,
    BSDF_TRANSMISSION = 2,
    BSDF_DIFFUSE = 4,
    BSDF_GLOSSY = 8,
    BSDF_SPECULAR = 16,
    BSDF_ALL = 31
};

BG_D float cos2_theta(V3 w) { return w.z * w.z; }
BG_D float abs_cos_theta(V3 w) { return fabsf(w.z); }
BG_D float sin2_theta(V3 w) { return rmax(0.0f, 1.0f - cos2_theta(w)); }
BG_D float sin_theta(V3 w) { return sqrtf(sin2_theta(w)); }
BG_D float tan_theta(V3 w) { return sin_theta(w) / w.z; }
BG_D float tan2_theta(V3 w) { return sin2_theta(w) / cos2_theta(w); }
BG_D float cos_phi(V3 w) {
    float v = sin_theta(w);
    return v == 0.0f ? 1.0f : rclamp(w.x / v, -1.0f, 1.0f);
}
BG_D float sin_phi(V3 w) {
    float v = sin_theta(w);
    return v == 0.0f ? 0.0f : rclamp(w.y / v, -1.0f, 1.0f);
}
BG_D float cos2_phi(V3 w) { return cos_phi(w) * cos_phi(w); }
BG_D float sin2_phi(V3 w) { return sin_phi(w) * sin_phi(w); }
BG_D bool same_hemisphere(V3 a, V3 b) { return a.z * b.z > 0.0f; }
BG_D V3 reflect(V3 wo, V3 n) { return -wo + 2.0f * dot(wo, n) * n; }
BG_D bool refract(V3 wi, V3 n, float eta, V3* wt) {  // bxdf.rs:146-159
    float ci = dot(n, wi);
    float s2i = rmax(0.0f, 1.0f - ci * ci);
    float s2t = eta * eta * s2i;
    if (s2t >= 1.0f) return false;
    float ct = sqrtf(1.0f - s2t);
    *wt = eta * -wi + (eta * ci - ct) * n;
    return true;
}
template <bool REF>
BG_D float fresnel_dielectric(float ci, float ei, float et) {  // bxdf.rs:165-188
    ci = rclamp(ci, -1.0f, 1.0f);
    if (!(ci > 0.0f)) {
        float t = ei;
        ei = et;
        et = t;
        if (!REF) ci = fabsf(ci);
    }
    float si = sqrtf(rmax(0.0f, 1.0f - ci * ci));
    float st = ei / et * si;
    if (st >= 1.0f) return 1.0f;
    float ct = sqrtf(rmax(0.0f, 1.0f - st * st));
    float rpar = ((et * ci) - (ei * ct)) / ((et * ci) + (ei * ct));
    float rperp = ((ei * ci) - (et * ct)) / ((ei * ci) + (et * ct));
    return (rpar * rpar + rperp * rperp) / 2.0f;
}
BG_D RGB fresnel_conductor(float cin, RGB eta_i, RGB eta_t, RGB k) {  // bxdf.rs:190-217
    RGB ci = rgb(rclamp(cin, -1.0f, 1.0f));
    RGB eta = eta_t / eta_i;
    RGB eta_k = k / eta_i;
    RGB ci2 = ci * ci;
    RGB si2 = rgb(1.0f) - ci2;
    RGB eta2 = eta * eta;
    RGB etak2 = eta_k * eta_k;
    RGB t0 = eta2 - etak2 - si2;
    RGB a2b2 = rgb_sqrt(t0 * t0 + eta2 * etak2 * 4.0f);
    RGB t1 = a2b2 + ci2;
    RGB a = rgb_sqrt((a2b2 + t0) * 0.5f);
    RGB t2 = ci * a * 2.0f;
    RGB rs = (t1 - t2) / (t1 + t2);
    RGB t3 = ci2 * a2b2 + si2 * si2;
    RGB t4 = t2 * si2;
    RGB rp = rs * (t3 - t4) / (t3 + t4);
    return (rp + rs) * 0.5f;
}

// TrowbridgeReitzDistribution (src/base/microfacet.rs), isotropic alpha.
struct TR {
    float ax, ay;
    BG_D float D(V3 wh) const {
        float t2 = tan2_theta(wh);
        if (isinf(t2)) return 0.0f;
        float cos4 = cos2_theta(wh) * cos2_theta(wh);
        float e = (cos2_phi(wh) / (ax * ax) + sin2_phi(wh) / (ay * ay)) * t2;
        return 1.0f / (PI * ax * ay * cos4 * (1.0f + e) * (1.0f + e));
    }
    BG_D float lambda(V3 w) const {
        float at = fabsf(tan_theta(w));
        if (isinf(at)) return 0.0f;
        float alpha = sqrtf(cos2_phi(w) * ax * ax + sin2_phi(w) * ay * ay);
        float a2t2 = (alpha * at) * (alpha * at);
        return (-1.0f + sqrtf(1.0f + a2t2)) / 2.0f;
    }
    template <bool REF>
    BG_D float G1(V3 w) const {  // F4
        return REF ? 1.0f / (1.0f / lambda(w)) : 1.0f / (1.0f + lambda(w));
    }
    BG_D float G(V3 wo, V3 wi) const { return 1.0f / (1.0f + lambda(wo) + lambda(wi)); }
    template <bool REF>
    BG_D float pdf(V3 wo, V3 wh) const { return D(wh) * G1<REF>(wo) * abs_dot(wo, wh) / abs_cos_theta(wo); }
    template <bool REF>
    BG_D static void sample11(float cos_t, float u1, float u2, float* sxo, float* syo) {  // :55-97
        if (cos_t > 0.9999f) {
            float r = sqrtf(u1 / (1.0f - u1));
            float phi = 6.28318530718f * u2;
            *sxo = r * cosf(phi);
            *syo = r * sinf(phi);
            return;
        }
        float sin_t = sqrtf(rmax(1.0f - cos_t * cos_t, 0.0f));
        float tan_t = sin_t / cos_t;
        float a = 1.0f / tan_t;
        float g1 = 2.0f / (1.0f + sqrtf(1.0f + 1.0f / (a * a)));
        float A = 2.0f * u1 / g1 - 1.0f;
        float tmp = 1.0f / (A * A - 1.0f);
        if (tmp > 1e10f) tmp = 1e10f;
        float B = tan_t;
        float D = sqrtf(rmax(B * B * tmp * tmp - (A * A - B * B) * tmp, 0.0f));
        float sx1 = B * tmp - D;
        float sx2 = B * tmp + D;
        float sx = REF ? sx1 : ((A < 0.0f || sx2 > 1.0f / tan_t) ? sx1 : sx2);  // F5
        float S;
        if (u2 > 0.5f) {
            S = 1.0f;
            u2 = 2.0f * (u2 - 0.5f);
        } else {
            S = -1.0f;
            u2 = 2.0f * (0.5f - u2);
        }
        float z = (u2 * (u2 * (u2 * 0.27385f - 0.73369f) + 0.46341f)) /
                  (u2 * (u2 * (u2 * 0.093073f + 0.309420f) - 1.000000f) + 0.597999f);
        *sxo = sx;
        *syo = S * z * sqrtf(1.0f + sx * sx);
    }
    template <bool REF>
    BG_D V3 sample_wh(V3 wo, float u0, float u1) const {  // :99-112, :144-153
        bool flip = wo.z < 0.0f;
        V3 wi = flip ? -wo : wo;
        V3 ws = normalize(v3(ax * wi.x, ay * wi.y, wi.z));
        float sx, sy;
        sample11<REF>(ws.z, u0, u1, &sx, &sy);
        float tmp = cos_phi(ws) * sx - sin_phi(ws) * sy;
        sy = sin_phi(ws) * sx + cos_phi(ws) * sy;
        sx = tmp;
        sx = ax * sx;
        sy = ay * sy;
        V3 wh = normalize(v3(-sx, -sy, 1.0f));
        return flip ? -wh : wh;
    }
};

// sampling.rs:181-198 / :238-242
BG_D V3 cosine_sample_hemisphere(float u0, float u1) {
    float ox = 2.0f * u0 - 1.0f, oy = 2.0f * u1 - 1.0f;
    float dx = 0.0f, dy = 0.0f;
    if (!(ox == 0.0f && oy == 0.0f)) {
        float theta, r;
        if (fabsf(ox) > fabsf(oy)) {
            theta = (PI / 4.0f) * (oy / ox);
            r = ox;
        } else {
            theta = PI_OVER_TWO - (PI / 4.0f) * (ox / oy);
            r = oy;
        }
        dx = r * cosf(theta);
        dy = r * sinf(theta);
    }
    float z = sqrtf(rmax(0.0f, 1.0f - dx * dx - dy * dy));
    return v3(dx, dy, z);
}
BG_D float power_heuristic(float nf, float fp, float ng, float gp) {
    float f = nf * fp, g = ng * gp;
    return (f * f) / (f * f + g * g);
}

// BX_OREN_NAYAR: src/bxdfs/oren_nayer.rs; BX_SPEC_REFL / BX_SPEC_TRANS: SpecularReflection /
// SpecularTransmission (src/bxdfs/specular.rs), the dielectric's two lobes when the caller does
// not allow a multi-lobe BxDF (the Whitted and direct-lighting integrators, PBRT mode).
enum BxKind : uint8_t {
    BX_LAMBERT = 0,
    BX_MF_REFL = 1,
    BX_FRESNEL_SPEC = 2,
    BX_OREN_NAYAR = 3,
    BX_SPEC_REFL = 4,
    BX_SPEC_TRANS = 5
};
struct Bxdf {
    uint8_t kind, type;
    bool conductor;
    RGB r;             // R (lambert, Oren-Nayar, microfacet, specular R / T)
    TR dist;
    RGB eta_t, k;      // conductor (eta_i = 1)
    float ei, et;      // dielectric fresnel / specular eta_a, eta_b; Oren-Nayar A, B
    BG_D bool matches(uint8_t f) const { return (type & f) == type; }
};
struct BxSample {
    V3 wi;
    RGB f;
    float pdf;
    int stype;
};

// Field-wise select of one of two BxDFs: keeps both in registers (indexing the pair with a runtime
// index would place it in local memory).
BG_D RGB sel(bool s, RGB a, RGB b) { return rgb(s ? b.r : a.r, s ? b.g : a.g, s ? b.b : a.b); }
BG_D Bxdf select_bxdf(bool second, const Bxdf& a, const Bxdf& b) {
    Bxdf r;
    r.kind = second ? b.kind : a.kind;
    r.type = second ? b.type : a.type;
    r.conductor = second ? b.conductor : a.conductor;
    r.r = sel(second, a.r, b.r);
    r.dist.ax = second ? b.dist.ax : a.dist.ax;
    r.dist.ay = second ? b.dist.ay : a.dist.ay;
    r.eta_t = sel(second, a.eta_t, b.eta_t);
    r.k = sel(second, a.k, b.k);
    r.ei = second ? b.ei : a.ei;
    r.et = second ? b.et : a.et;
    return r;
}

// OrenNayer::f (oren_nayer.rs:34-60)
BG_D RGB oren_nayar_f(const Bxdf& b, V3 wo, V3 wi) {
    float sti = sin_theta(wi), sto = sin_theta(wo);
    float max_cos = 0.0f;
    if (sti > 1e-4f && sto > 1e-4f) {
        float spi = sin_phi(wi), cpi = cos_phi(wi), spo = sin_phi(wo), cpo = cos_phi(wo);
        max_cos = rmax(0.0f, cpi * cpo + spi * spo);
    }
    float sin_alpha, tan_beta;
    if (abs_cos_theta(wi) > abs_cos_theta(wo)) {
        sin_alpha = sto;
        tan_beta = sti / abs_cos_theta(wi);
    } else {
        sin_alpha = sti;
        tan_beta = sto / abs_cos_theta(wo);
    }
    return b.r * (1.0f / PI) * (b.ei + b.et * max_cos * sin_alpha * tan_beta);
}

template <bool REF>
BG_D RGB bx_f(const Bxdf& b, V3 wo, V3 wi) {
    if (b.kind == BX_LAMBERT) return b.r * (1.0f / PI);
    if (b.kind == BX_OREN_NAYAR) return oren_nayar_f(b, wo, wi);
    if (b.kind == BX_MF_REFL) {  // bxdfs/microfacet.rs:69-94
        float co = abs_cos_theta(wo), ci = abs_cos_theta(wi);
        V3 wh = wi + wo;
        if (ci == 0.0f || co == 0.0f) return rgb(0.0f);
        if (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) return rgb(0.0f);
        wh = normalize(wh);
        float c = dot(wi, face_forward(wh, v3(0.0f, 0.0f, 1.0f)));
        RGB F = b.conductor ? fresnel_conductor(fabsf(c), rgb(1.0f), b.eta_t, b.k)
                            : rgb(fresnel_dielectric<REF>(c, b.ei, b.et));
        return b.r * b.dist.D(wh) * b.dist.G(wo, wi) * F / (4.0f * ci * co);
    }
    return rgb(0.0f);
}
template <bool REF>
BG_D float bx_pdf(const Bxdf& b, V3 wo, V3 wi) {
    if (b.kind == BX_LAMBERT || b.kind == BX_OREN_NAYAR)
        return same_hemisphere(wo, wi) ? abs_cos_theta(wi) * (1.0f / PI) : 0.0f;
    if (b.kind == BX_MF_REFL) {
        if (!same_hemisphere(wo, wi)) return 0.0f;
        V3 wh = normalize(wo + wi);
        return b.dist.pdf<REF>(wo, wh) / (4.0f * dot(wo, wh));
    }
    return 0.0f;
}
template <bool REF>
BG_D BxSample bx_sample(const Bxdf& b, V3 wo, float u0, float u1) {
    BxSample s;
    s.wi = v3(0, 0, 0);
    s.f = rgb(0.0f);
    s.pdf = 0.0f;
    s.stype = -1;
    if (b.kind == BX_LAMBERT || b.kind == BX_OREN_NAYAR) {
        V3 wi = cosine_sample_hemisphere(u0, u1);
        if (wo.z < 0.0f) wi.z *= -1.0f;
        s.wi = wi;
        s.f = bx_f<REF>(b, wo, wi);
        s.pdf = bx_pdf<REF>(b, wo, wi);
        return s;
    }
    if (b.kind == BX_MF_REFL) {
        if (wo.z == 0.0f) return s;
        V3 wh = b.dist.sample_wh<REF>(wo, u0, u1);
        if (dot(wo, wh) < 0.0f) return s;
        V3 wi = reflect(wo, wh);
        if (!same_hemisphere(wo, wi)) return s;
        s.wi = wi;
        s.f = bx_f<REF>(b, wo, wi);
        s.pdf = b.dist.pdf<REF>(wo, wh) / (4.0f * dot(wo, wh));
        return s;
    }
    if (b.kind == BX_SPEC_REFL) {  // specular.rs:57-66
        V3 wi = v3(-wo.x, -wo.y, wo.z);
        s.wi = wi;
        s.f = rgb(fresnel_dielectric<REF>(wi.z, b.ei, b.et)) * b.r / abs_cos_theta(wi);
        s.pdf = 1.0f;
        return s;
    }
    if (b.kind == BX_SPEC_TRANS) {  // specular.rs:82-113
        bool entering = wo.z > 0.0f;
        float ei = entering ? b.ei : b.et, et = entering ? b.et : b.ei;
        V3 wi;
        if (!refract(wo, face_forward(v3(0.0f, 0.0f, 1.0f), wo), ei / et, &wi)) return s;
        RGB f = b.r * (rgb(1.0f) - rgb(fresnel_dielectric<REF>(wi.z, b.ei, b.et)));
        f = f * ((ei * ei) / (et * et));
        s.wi = wi;
        s.f = f / abs_cos_theta(wi);
        s.pdf = 1.0f;
        return s;
    }
    // FresnelSpecular (bxdfs/fresnel.rs:76-122)
    float F = fresnel_dielectric<REF>(wo.z, b.ei, b.et);
    if (u0 < F) {
        V3 wi = v3(-wo.x, -wo.y, wo.z);
        s.wi = wi;
        s.pdf = F;
        s.f = rgb(F) * b.r / abs_cos_theta(wi);
        s.stype = BSDF_SPECULAR | BSDF_REFLECTION;
        return s;
    }
    bool entering = wo.z > 0.0f;
    float ei = entering ? b.ei : b.et, et = entering ? b.et : b.ei;
    V3 wi;
    if (!refract(wo, face_forward(v3(0.0f, 0.0f, 1.0f), wo), ei / et, &wi)) return s;
    RGB ft = b.r * (1.0f - F);  // T = R = 1 for the dielectric
    ft = ft * ((ei * ei) / (et * et));
    s.wi = wi;
    s.f = ft / abs_cos_theta(wi);
    s.pdf = 1.0f - F;
    s.stype = BSDF_SPECULAR | BSDF_TRANSMISSION;
    return s;
}

// BSDF (src/base/bsdf.rs) with at most two lobes in fixed slots: slot 0 holds the first BxDF the
// material adds, slot 1 the second.  Loops run over both slots with compile-time indices (guarded
// by n) so the lobes stay in registers; the iteration order is the reference's insertion order.
struct BSDF {
    float eta;
    V3 ns, ng, ss, ts;
    Bxdf bx[2];
    int n;
    BG_D int num_components(uint8_t f) const {
        int k = 0;
#pragma unroll
        for (int i = 0; i < 2; ++i)
            if (i < n) k += bx[i].matches(f);
        return k;
    }
    BG_D V3 to_local(V3 v) const { return v3(dot(v, ss), dot(v, ts), dot(v, ns)); }
    BG_D V3 to_world(V3 v) const {
        return v3(ss.x * v.x + ts.x * v.y + ns.x * v.z, ss.y * v.x + ts.y * v.y + ns.y * v.z,
                  ss.z * v.x + ts.z * v.y + ns.z * v.z);
    }
    template <bool REF>
    BG_D RGB f(V3 wo_w, V3 wi_w, uint8_t flags) const {  // bsdf.rs:84-105
        V3 wo = to_local(wo_w), wi = to_local(wi_w);
        if (wo.z == 0.0f) return rgb(0.0f);
        bool refl = dot(wi_w, ng) * dot(wo_w, ng) > 0.0f;
        RGB r = rgb(0.0f);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            if (i < n && bx[i].matches(flags) &&
                ((refl && (bx[i].type & BSDF_REFLECTION)) || (!refl && (bx[i].type & BSDF_TRANSMISSION))))
                r = r + bx_f<REF>(bx[i], wo, wi);
        return r;
    }
    template <bool REF>
    BG_D float pdf(V3 wo_w, V3 wi_w, uint8_t flags) const {  // bsdf.rs:234-259
        if (n == 0) return 0.0f;
        V3 wo = to_local(wo_w), wi = to_local(wi_w);
        if (wo.z == 0.0f) return 0.0f;
        float ret = 0.0f, comps = 0.0f;
#pragma unroll
        for (int i = 0; i < 2; ++i)
            if (i < n && bx[i].matches(flags)) {
                comps += 1.0f;
                ret += bx_pdf<REF>(bx[i], wo, wi);
            }
        return comps > 0.0f ? ret / comps : 0.0f;
    }
    template <bool REF>
    BG_D BxSample sample(V3 wo_w, float u0, float u1, uint8_t type) const {  // bsdf.rs:140-232
        BxSample zero;
        zero.wi = v3(0, 0, 0);
        zero.f = rgb(0.0f);
        zero.pdf = 0.0f;
        zero.stype = 0;
        int matches = num_components(type);
        if (matches == 0) return zero;
        uint32_t comp = min((uint32_t)floorf(u0 * (float)matches), (uint32_t)matches - 1);
        uint32_t count = comp;
        int pick = -1;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            if (pick < 0 && i < n) {
                if (bx[i].matches(type) && count == 0) pick = i;
                else if (REF || bx[i].matches(type)) count -= 1;  // F8
            }
        }
        if (pick < 0) return zero;
        const Bxdf b = select_bxdf(pick != 0, bx[0], bx[1]);
        float ur0 = rmin(u0 * (float)matches - (float)comp, ONE_MINUS_EPSILON);
        V3 wo = to_local(wo_w);
        if (wo.z == 0.0f) return zero;
        BxSample s = bx_sample<REF>(b, wo, ur0, u1);
        int stype = s.stype >= 0 ? s.stype : b.type;
        if (s.pdf == 0.0f) return zero;
        V3 wi_w = to_world(s.wi);
        if (!(b.type & BSDF_SPECULAR) && matches > 1) {
#pragma unroll
            for (int i = 0; i < 2; ++i)
                if (i < n && i != pick && bx[i].matches(type)) s.pdf += bx_pdf<REF>(bx[i], wo, s.wi);
        }
        if (matches > 1) s.pdf /= (float)matches;
        if (!(b.type & BSDF_SPECULAR)) {
            bool refl = dot(wi_w, ng) * dot(wo_w, ng) > 0.0f;
            s.f = rgb(0.0f);
#pragma unroll
            for (int i = 0; i < 2; ++i)
                if (i < n && bx[i].matches(type) &&
                    ((refl && (bx[i].type & BSDF_REFLECTION)) || (!refl && (bx[i].type & BSDF_TRANSMISSION))))
                    s.f = s.f + bx_f<REF>(bx[i], wo, s.wi);
        }
        s.wi = wi_w;
        s.stype = stype;
        return s;
    }
};

BG_D uint32_t prim_material(const Scene& sc, int prim) {
    if ((uint32_t)prim < sc.ntri) return __float_as_uint(sc.tri[3 * prim].w);
    if ((uint32_t)prim < sc.ntri + sc.nsph) return sc.sph_mat[prim - sc.ntri];
    return __float_as_uint(sc.quads[QUADRIC_F4 * (prim - sc.ntri - sc.nsph) + 7].w);
}

BG_D bool material_textured(const Material& m) { return (m.kd_tex | m.ks_tex) != 0u; }
BG_D RGB clamp_rgb0(RGB c) {  // RGBSpectrum::clamp(0, +inf)
    return rgb(rclamp(c.r, 0.0f, INFINITY), rclamp(c.g, 0.0f, INFINITY), rclamp(c.b, 0.0f, INFINITY));
}

// Material::compute_scattering_functions (src/materials/{matte,plastic}.rs and the composed
// conductor / dielectric).  CLS is the material type when the caller knows it (the wavefront
// shades one material class per launch), -1 to read it from the record.  `tp` carries the
// texture inputs (needed when the material is textured); `multi_lobe` = allow_multiple_lobes:
// false splits the dielectric into SpecularReflection + SpecularTransmission in PBRT mode.
template <int CLS = -1, bool REF = false>
BG_D BSDF make_bsdf(const Scene& sc, const Isect& it, const TexPoint* tp = nullptr, bool multi_lobe = true) {
    const Material& m = sc.mats[prim_material(sc, it.prim)];
    const uint32_t type = CLS >= 0 ? (uint32_t)CLS : m.type;
    BSDF b;
    b.eta = 1.0f;
    b.n = 0;
    b.ns = it.ns;
    b.ng = it.n;
    b.ss = normalize(it.dpdu);
    b.ts = cross(b.ns, b.ss);
    if (type == 0 || type == 1) {  // matte, plastic
        // Lambertian / Oren-Nayar (if kd != 0) then glossy (plastic, if ks != 0), packed into the
        // fixed slots with selects: a slot chosen by a runtime index would force the BSDF into
        // local memory.
        RGB kd = (m.kd_tex && tp) ? tex_eval<REF>(sc, m.kd_tex - 1u, *tp) : rgb(m.kd[0], m.kd[1], m.kd[2]);
        kd = clamp_rgb0(kd);
        Bxdf l{};
        const bool oren = type == 0 && m.sigma != 0.0f;
        l.kind = oren ? BX_OREN_NAYAR : BX_LAMBERT;
        l.type = BSDF_REFLECTION | BSDF_DIFFUSE;
        l.r = kd;
        l.conductor = false;
        l.ei = m.on_a;
        l.et = m.on_b;
        const bool has_l = !is_black(kd);
        bool has_g = false;
        Bxdf g{};
        if (type == 1) {
            RGB ks = (m.ks_tex && tp) ? tex_eval<REF>(sc, m.ks_tex - 1u, *tp) : rgb(m.ks[0], m.ks[1], m.ks[2]);
            ks = clamp_rgb0(ks);
            has_g = !is_black(ks);
            g.kind = BX_MF_REFL;
            g.type = BSDF_REFLECTION | BSDF_GLOSSY;
            g.r = ks;
            g.dist = TR{m.alpha, m.alpha};
            g.conductor = false;
            g.ei = 1.5f;
            g.et = 1.0f;
        }
        b.bx[0] = select_bxdf(!has_l, l, g);
        b.bx[1] = g;
        b.n = (has_l ? 1 : 0) + (has_g ? 1 : 0);
    } else if (type == 2) {  // conductor
        Bxdf& g = b.bx[b.n++];
        g.kind = BX_MF_REFL;
        g.type = BSDF_REFLECTION | BSDF_GLOSSY;
        g.r = rgb(1.0f);
        g.dist = TR{m.alpha, m.alpha};
        g.conductor = true;
        g.eta_t = rgb(m.eta[0], m.eta[1], m.eta[2]);
        g.k = rgb(m.k[0], m.k[1], m.k[2]);
    } else if (REF || multi_lobe) {  // dielectric
        b.eta = m.ior;
        Bxdf& d = b.bx[b.n++];
        d.kind = BX_FRESNEL_SPEC;
        d.type = BSDF_REFLECTION | BSDF_TRANSMISSION | BSDF_SPECULAR;
        d.r = rgb(1.0f);
        d.conductor = false;
        d.ei = 1.0f;
        d.et = m.ior;
    } else {  // dielectric as two specular lobes (PBRT-v3 GlassMaterial without multiple lobes)
        b.eta = m.ior;
        Bxdf r{}, t{};
        r.kind = BX_SPEC_REFL;
        r.type = BSDF_REFLECTION | BSDF_SPECULAR;
        r.r = rgb(1.0f);
        r.ei = 1.0f;
        r.et = m.ior;
        t.kind = BX_SPEC_TRANS;
        t.type = BSDF_TRANSMISSION | BSDF_SPECULAR;
        t.r = rgb(1.0f);
        t.ei = 1.0f;
        t.et = m.ior;
        b.bx[0] = r;
        b.bx[1] = t;
        b.n = 2;
    }
    return b;
}

// ---- lights (src/lights/diffuse.rs)
BG_D RGB emission(const Emission& e, V3 n, V3 dir) {
    if (e.two_sided || dot(n, dir) > 0.0f) return rgb(e.intensity[0], e.intensity[1], e.intensity[2]);
    return rgb(0.0f);
}
BG_D int prim_emission(const Scene& sc, int prim) {
    if (prim < 0) return -1;
    if ((uint32_t)prim < sc.ntri) return __float_as_int(sc.tri[3 * prim + 1].w);
    if ((uint32_t)prim < sc.ntri + sc.nsph) return sc.sph_emis ? sc.sph_emis[prim - sc.ntri] : -1;
    return sc.quad_emis ? sc.quad_emis[prim - sc.ntri - sc.nsph] : -1;
}
BG_D RGB emitted_radiance(const Scene& sc, const Isect& it, V3 w) {  // interaction.rs:257-266
    int e = prim_emission(sc, it.prim);
    if (e < 0) return rgb(0.0f);
    return emission(sc.emis[e], it.n, w);
}

struct LightSample {
    RGB radiance;
    V3 wi;
    float pdf;
    ShapeSample pt;
};

// ---- shapes as area lights: Shape::sample (sphere.rs:328-355, disk.rs:184-214, cylinder.rs:289-321)
// and area (sphere.rs:375-377, disk.rs:216-218, cylinder.rs:323-325).  Spheres are full with a
// translation-only transform; quadrics carry their affine transform (rows 0-2 object-to-world,
// rows 3-5 world-to-object).
BG_D float sphere_area(float r) { return (360.0f * (PI / 180.0f)) * r * (r - (-r)); }
BG_D float quadric_area(const float4* q) {
    const float4 p0 = q[6], p1 = q[7];
    const int kind = (int)(__float_as_uint(p1.z) & 0xFFu);
    if (kind == 1) return p1.y * 0.5f * (p0.x * p0.x - p0.y * p0.y);  // disk
    return (p0.w - p0.z) * p0.x * p1.y;                                // cylinder
}
// Sphere::sample.  REF (F21): the normal is the object-space point itself, not normalised (length
// radius), so Shape::sample_from_it's |cos| and pdf carry a factor radius.
template <bool REF>
BG_D ShapeSample sphere_light_sample(float4 s, float u0, float u1) {
    const float r = s.w;
    const float z = 1.0f - 2.0f * u0;  // uniform_sample_sphere (sampling.rs:211-216)
    const float rr = sqrtf(rmax(1.0f - z * z, 0.0f));
    const float phi = 2.0f * PI * u1;
    V3 obj = v3(0.0f + r * (rr * cosf(phi)), 0.0f + r * (rr * sinf(phi)), 0.0f + r * z);
    ShapeSample ss;
    ss.n = REF ? obj : normalize(obj);
    const float k = r / length(obj);  // reprojection onto the surface
    obj = v3(obj.x * k, obj.y * k, obj.z * k);
    const V3 oerr = gamma(5.0f) * vabs(obj);
    M34 t;
    t.m[0][0] = 1.0f; t.m[0][1] = 0.0f; t.m[0][2] = 0.0f; t.m[0][3] = s.x;
    t.m[1][0] = 0.0f; t.m[1][1] = 1.0f; t.m[1][2] = 0.0f; t.m[1][3] = s.y;
    t.m[2][0] = 0.0f; t.m[2][1] = 0.0f; t.m[2][2] = 1.0f; t.m[2][3] = s.z;
    ss.p = m_point_perr(t, obj, oerr, &ss.p_err);
    ss.pdf_area = 1.0f / sphere_area(r);
    ss.b0 = ss.b1 = 0.0f;
    return ss;
}
// Disk::sample / Cylinder::sample.  REF (F22): the disk draws from the whole disk of the outer
// radius whatever inner_radius and phi_max (the intersection-based pdf is 0 in the hole), and the
// cylinder's normal is not normalised (F21).  PBRT draws the annulus sector uniformly and
// normalises.
template <bool REF>
BG_D ShapeSample quadric_light_sample(const float4* q, float u0, float u1) {
    const float4 p0 = q[6], p1 = q[7];
    const uint32_t flags = __float_as_uint(p1.z);
    const int kind = (int)(flags & 0xFFu);
    const bool reverse = (flags >> 8) & 1u;
    const float radius = p0.x, inner = p0.y, z_min = p0.z, z_max = p0.w, height = p1.x, phi_max = p1.y;
    const M34 o2w = load_m34(q), w2o = load_m34(q + 3);
    ShapeSample ss;
    V3 obj, oerr = v3(0.0f, 0.0f, 0.0f);
    if (kind == 1) {
        if (REF) {
            const float2 d = concentric_sample_disk(u0, u1);
            obj = v3(d.x * radius, d.y * radius, height);
        } else {
            const float rad = sqrtf((1.0f - u0) * (inner * inner) + u0 * (radius * radius));
            const float ph = u1 * phi_max;
            obj = v3(rad * cosf(ph), rad * sinf(ph), height);
        }
        ss.n = normalize(m_normal(w2o, v3(0.0f, 0.0f, 1.0f)));
    } else {
        const float z = (1.0f - u0) * z_min + u0 * z_max;  // lerp (math.rs:7-9)
        const float phi = u1 * phi_max;
        obj = v3(radius * cosf(phi), radius * sinf(phi), z);
        const V3 n = m_normal(w2o, v3(obj.x, obj.y, 0.0f));
        ss.n = REF ? n : normalize(n);
        const float hr = sqrtf(obj.x * obj.x + obj.y * obj.y);
        obj.x *= radius / hr;
        obj.y *= radius / hr;
        oerr = gamma(3.0f) * vabs(v3(obj.x, obj.y, 0.0f));
    }
    if (reverse) ss.n = ss.n * -1.0f;
    ss.p = m_point_perr(o2w, obj, oerr, &ss.p_err);
    ss.pdf_area = 1.0f / quadric_area(q);
    ss.b0 = ss.b1 = 0.0f;
    return ss;
}

// DiffuseAreaLight::sample_point + Shape::sample_from_it (diffuse.rs:54-87, shape.rs:17-34) for a
// triangle, sphere, disk or cylinder light (SHAPES = false: triangles only, for light lists that
// hold nothing else).
template <bool REF, bool SHAPES = true>
BG_D LightSample light_sample(const Scene& sc, uint32_t prim, const Isect& it, float u0, float u1) {
    LightSample ls;
    ls.radiance = rgb(0.0f);
    ls.wi = v3(0, 0, 0);
    ls.pdf = 0.0f;
    if (!SHAPES || prim < sc.ntri) {
        V3 p0, p1, p2;
        load_tri(sc, prim, &p0, &p1, &p2);
        ls.pt = tri_sample(p0, p1, p2, u0, u1);
        if (tri_flag_bits(sc, prim) & TRI_SFLIP) ls.pt.n = ls.pt.n * -1.0f;
    } else if (prim < sc.ntri + sc.nsph) {
        ls.pt = sphere_light_sample<REF>(sc.sph[prim - sc.ntri], u0, u1);
    } else {
        ls.pt = quadric_light_sample<REF>(sc.quads + QUADRIC_F4 * (prim - sc.ntri - sc.nsph), u0, u1);
    }
    V3 wi = ls.pt.p - it.p;
    float pdf;
    if (length_squared(wi) == 0.0f) pdf = 0.0f;
    else {
        wi = normalize(wi);
        float conv = distance_squared(it.p, ls.pt.p) / abs_dot(ls.pt.n, -wi);
        pdf = REF ? conv : ls.pt.pdf_area * conv;  // F13
        if (isinf(pdf)) pdf = 0.0f;
    }
    if (pdf == 0.0f || length_squared(ls.pt.p - it.p) == 0.0f) return ls;
    ls.wi = normalize(ls.pt.p - it.p);
    ls.radiance = emission(sc.emis[prim_emission(sc, (int)prim)], ls.pt.n, REF ? ls.wi : -ls.wi);  // F12
    ls.pdf = pdf;
    return ls;
}
// Shape::pdf_from_it (shape.rs:40-57) of a triangle, sphere, disk or cylinder light.  Also returns
// the hit distance and the light's surface normal there (for its one-sided emission).  REF (F20):
// a sphere seen from outside reports the pdf of uniform cone sampling (sphere.rs:357-373),
// although Sphere::sample draws uniformly by area.
template <bool REF, bool SHAPES = true>
BG_D float light_pdf(const Scene& sc, uint32_t prim, const Isect& it, V3 wi, float* t_light, V3* n_light = nullptr) {
    Ray ray = spawn_ray(it.p, it.p_err, it.n, it.time, wi, REF);
    Isect li;
    float area, t;
    if (!SHAPES || prim < sc.ntri) {
        V3 p0, p1, p2;
        load_tri(sc, prim, &p0, &p1, &p2);
        TriRay tr = make_tri_ray(ray);
        TriHit h;
        if (!tri_test(tr, ray.t_max, p0, p1, p2, &h)) return 0.0f;
        tri_isect_plain(p0, p1, p2, h, ray, &li);
        if (tri_flag_bits(sc, prim) & TRI_LFLIP) li.n = -li.n;
        area = tri_area(p0, p1, p2);
        t = h.t;
    } else if (prim < sc.ntri + sc.nsph) {
        const float4 s = sc.sph[prim - sc.ntri];
        if (REF) {
            const V3 center = v3(s.x, s.y, s.z);
            const V3 o = offset_ray_origin(it.p, it.p_err, it.n, center - it.p);
            if (!(distance_squared(o, center) <= s.w * s.w)) {
                const float sin2 = s.w * s.w / distance_squared(it.p, center);
                const float cos_max = sqrtf(rmax(0.0f, 1.0f - sin2));
                if (t_light) *t_light = INFINITY;
                return 1.0f / (2.0f * PI * (1.0f - cos_max));  // uniform_cone_pdf
            }
        }
        SphHit h;
        if (!sphere_test(s, ray, ray.t_max, &h)) return 0.0f;
        sphere_isect(s, h, ray, &li);
        area = sphere_area(s.w);
        t = h.t;
    } else {
        const float4* q = sc.quads + QUADRIC_F4 * (prim - sc.ntri - sc.nsph);
        if (!quadric_hit(q, ray, ray.t_max, &t, &li)) return 0.0f;
        area = quadric_area(q);
    }
    float pdf = distance_squared(it.p, li.p) / (abs_dot(li.n, -wi) * area);
    if (isinf(pdf)) pdf = 0.0f;
    if (t_light) *t_light = t;
    if (n_light) *n_light = li.n;
    return pdf;
}

// ---- InfiniteAreaLight (src/lights/infinite.rs) and Distribution2D (src/base/sampling.rs:10-118)
BG_D V3 m34_vec(const float m[3][4], V3 v) {  // Vec3::transform with an affine 3x4
    return v3(m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z, m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z,
              m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z);
}
// find_interval (src/base/math.rs:70-87) over a cdf of `size` entries
BG_D uint32_t find_interval(const float* cdf, uint32_t size, float u) {
    uint32_t first = 0, len = size;
    while (len > 0) {
        uint32_t half = len >> 1, middle = first + half;
        if (cdf[middle] <= u) {
            first = middle + 1;
            len -= half + 1;
        } else {
            len = half;
        }
    }
    int32_t r = (int32_t)first - 1;
    return (uint32_t)(r < 0 ? 0 : (r > (int32_t)size - 2 ? (int32_t)size - 2 : r));
}
// find_interval through a guide table of g (a power of two) buckets: the same index, since the
// answer is monotone in u and k / g <= u < (k + 1) / g for k = floor(u * g) (exact in f32); every
// index up to the answer has cdf <= u, so the last such index in [guide[k], guide[k + 1]] is it.
BG_D uint32_t find_interval_guided(const float* cdf, float u, const uint32_t* guide, uint32_t g) {
    const float x = u * (float)g;
    uint32_t k = x >= (float)g ? g - 1 : (x > 0.0f ? (uint32_t)x : 0u);
    uint32_t lo = guide[k], hi = guide[k + 1];
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (cdf[mid] <= u) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}
// Distribution1D::sample_continuous (sampling.rs:53-76); `count` is the divisor of the result;
// `guide` (g buckets) accelerates the interval search.
BG_D float dist1d_sample(const float* cdf, const float* func, float func_int, uint32_t n, uint32_t count, float u,
                         float* pdf, uint32_t* off, const uint32_t* guide = nullptr, uint32_t g = 0) {
    uint32_t o = guide ? find_interval_guided(cdf, u, guide, g) : find_interval(cdf, n + 1, u);
    if (off) *off = o;
    float du = u - cdf[o];
    if (cdf[o + 1] - cdf[o] > 0.0f) du /= cdf[o + 1] - cdf[o];
    *pdf = func_int > 0.0f ? func[o] / func_int : 0.0f;
    return ((float)o + du) / (float)count;
}
// Distribution2D::sample_continuous (sampling.rs:99-111).  REF (F18): a conditional row keeps the
// whole tail of the function (sampling.rs:84), so its count() is (nv - v) * nu.
template <bool REF>
BG_D float2 dist2d_sample(const InfLight& L, float u0, float u1, float* pdf) {
    float p0, p1;
    uint32_t v = 0;
    const float d1 = dist1d_sample(L.marg_cdf, L.marg_func, L.marg_int, L.nv, L.nv, u1, &p1, &v, L.marg_guide, L.gv);
    const uint32_t count = REF ? (L.nv - v) * L.nu : L.nu;
    const float d0 = dist1d_sample(L.cond_cdf + (size_t)v * (L.nu + 1), L.cond_func + (size_t)v * L.nu,
                                   L.cond_int[v], L.nu, count, u0, &p0, nullptr, L.cond_guide + (size_t)v * (L.gu + 1),
                                   L.gu);
    *pdf = p0 * p1;
    return make_float2(d0, d1);
}
// Distribution2D::pdf (sampling.rs:113-117).  REF (F19): p is cast to an integer before the scaling,
// so the cell is (0, 0) unless a coordinate reaches 1; the column bound is row 0's count, the whole
// function (F18).  Row v's tail is the function from v * nu on; an index past its end (where the
// reference panics) reads the last entry.
template <bool REF>
BG_D float dist2d_pdf(const InfLight& L, float p0, float p1) {
    size_t idx;
    if (REF) {
        const size_t v = p1 >= 1.0f ? L.nv - 1 : 0;
        const size_t u = p0 >= 1.0f ? (size_t)L.nv * L.nu - 1 : 0;
        idx = v * L.nu + u;
        if (idx > (size_t)L.nv * L.nu - 1) idx = (size_t)L.nv * L.nu - 1;
    } else {
        int iu = (int)(p0 * (float)L.nu), iv = (int)(p1 * (float)L.nv);
        iu = iu < 0 ? 0 : (iu > (int)L.nu - 1 ? (int)L.nu - 1 : iu);
        iv = iv < 0 ? 0 : (iv > (int)L.nv - 1 ? (int)L.nv - 1 : iv);
        idx = (size_t)iv * L.nu + (size_t)iu;
    }
    return L.cond_func[idx] / L.marg_int;
}
// InfiniteAreaLight::radiance (infinite.rs:88-96): the map at the ray direction, level 0.
BG_D RGB inf_radiance(const Scene& sc, V3 dir) {
    const InfLight& L = *sc.inf;
    V3 w = normalize(m34_vec(L.w2l, dir));
    float phi = atan2f(w.y, w.x);
    if (phi < 0.0f) phi = phi + 2.0f * PI;
    float theta = acosf(rclamp(w.z, -1.0f, 1.0f));
    float2 st = make_float2(phi * (1.0f / (2.0f * PI)), theta * (1.0f / PI));
    return mip_filter(sc, L.map, st, make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f));
}
// InfiniteAreaLight::sample_point (infinite.rs:98-153); the visibility target is 2 world radii
// along wi with no error bound and no normal.
template <bool REF>
BG_D LightSample inf_sample(const Scene& sc, const Isect& it, float u0, float u1) {
    const InfLight& L = *sc.inf;
    LightSample ls;
    ls.radiance = rgb(0.0f);
    ls.wi = v3(0, 0, 0);
    ls.pdf = 0.0f;
    float map_pdf;
    float2 uv = dist2d_sample<REF>(L, u0, u1, &map_pdf);
    if (map_pdf == 0.0f) return ls;
    float theta = uv.y * PI, phi = uv.x * 2.0f * PI;
    float st = sinf(theta), ct = cosf(theta), sp = sinf(phi), cp = cosf(phi);
    V3 wi = m34_vec(L.l2w, v3(st * cp, st * sp, ct));
    float pdf = map_pdf / (2.0f * PI * PI * st);
    if (st == 0.0f) pdf = 0.0f;
    ls.wi = wi;
    ls.pdf = pdf;
    ls.radiance = mip_filter(sc, L.map, uv, make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f));
    ls.pt.p = it.p + wi * (2.0f * L.radius);
    ls.pt.p_err = v3(0.0f, 0.0f, 0.0f);
    ls.pt.n = v3(0.0f, 0.0f, 0.0f);
    ls.pt.pdf_area = 0.0f;
    return ls;
}
// InfiniteAreaLight::point_pdf (infinite.rs:155-169)
template <bool REF>
BG_D float inf_pdf(const Scene& sc, V3 w) {
    const InfLight& L = *sc.inf;
    V3 wi = m34_vec(L.w2l, w);
    float theta = acosf(rclamp(wi.z, -1.0f, 1.0f));
    float phi = atan2f(wi.y, wi.x);
    if (phi < 0.0f) phi = phi + 2.0f * PI;
    float s = sinf(theta);
    if (s == 0.0f) return 0.0f;
    return dist2d_pdf<REF>(L, phi * (1.0f / (2.0f * PI)), theta * (1.0f / PI)) / (2.0f * PI * PI * s);
}
// Light::sample_point for an entry of the light list (a triangle or the infinite light).
template <bool REF, bool SHAPES = true>
BG_D LightSample light_sample_any(const Scene& sc, uint32_t light, const Isect& it, float u0, float u1) {
    if (light == LIGHT_INFINITE) return inf_sample<REF>(sc, it, u0, u1);
    return light_sample<REF, SHAPES>(sc, light, it, u0, u1);
}
// Light::point_pdf for an entry of the light list.  t_light: the hit distance on an area light,
// infinity for the infinite light; n_light: the area light's normal there.
template <bool REF, bool SHAPES = true>
BG_D float light_pdf_any(const Scene& sc, uint32_t light, const Isect& it, V3 wi, float* t_light,
                         V3* n_light = nullptr) {
    if (light == LIGHT_INFINITE) {
        if (t_light) *t_light = INFINITY;
        return inf_pdf<REF>(sc, wi);
    }
    return light_pdf<REF, SHAPES>(sc, light, it, wi, t_light, n_light);
}
// Radiance arriving along a BSDF-sampled direction wi that reaches light `light` unoccluded:
// the area light's one-sided emission at its surface, or the environment map.
BG_D RGB light_radiance_along(const Scene& sc, uint32_t light, V3 wi, V3 n_light) {
    if (light == LIGHT_INFINITE) return inf_radiance(sc, wi);
    return emission(sc.emis[prim_emission(sc, (int)light)], n_light, -wi);
}
// Whether a scene's light list holds more than triangles (the infinite light, emitting spheres or
// quadrics): such scenes run the shade variants with the general light code.
BG_HD bool general_lights(const Scene& sc) { return sc.inf || sc.sph_emis || sc.quad_emis; }
// Light::radiance of every light for a ray that escapes the scene (only infinite lights emit).
BG_D RGB escaped_radiance(const Scene& sc, V3 dir) { return sc.inf ? inf_radiance(sc, dir) : rgb(0.0f); }

// ---- camera
BG_D V3 xf_point(const float m[4][4], V3 p) {  // point3.rs:51-69
    float xp = m[0][0] * p.x + m[0][1] * p.y + m[0][2] * p.z + m[0][3];
    float yp = m[1][0] * p.x + m[1][1] * p.y + m[1][2] * p.z + m[1][3];
    float zp = m[2][0] * p.x + m[2][1] * p.y + m[2][2] * p.z + m[2][3];
    float wp = m[3][0] * p.x + m[3][1] * p.y + m[3][2] * p.z + m[3][3];
    if (wp == 1.0f) return v3(xp, yp, zp);
    return v3(xp, yp, zp) / wp;
}
// PerspectiveCamera::generate_ray, pinhole (perspective.rs:117-175) + Ray::transform (ray.rs:50-76)
// lu0, lu1: the lens sample (used when c.lens_radius > 0).
BG_D Ray camera_ray(const Camera& c, float fx, float fy, float tu, float lu0 = 0.5f, float lu1 = 0.5f) {
    V3 cp = xf_point(c.r2c, v3(fx, fy, 0.0f));
    V3 d = normalize(cp);
    V3 oc = v3(0.0f, 0.0f, 0.0f);
    if (c.lens_radius > 0.0f) thin_lens(c, d, lu0, lu1, &oc, &d);
    const auto& m = c.c2w;
    float x = oc.x, y = oc.y, z = oc.z;
    float xp = (m[0][0] * x + m[0][1] * y) + (m[0][2] * z + m[0][3]);
    float yp = (m[1][0] * x + m[1][1] * y) + (m[1][2] * z + m[1][3]);
    float zp = (m[2][0] * x + m[2][1] * y) + (m[2][2] * z + m[2][3]);
    float wp = (m[3][0] * x + m[3][1] * y) + (m[3][2] * z + m[3][3]);
    float xa = fabsf(m[0][0] * x) + fabsf(m[0][1] * y) + fabsf(m[0][2] * z) + fabsf(m[0][3]);
    float ya = fabsf(m[1][0] * x) + fabsf(m[1][1] * y) + fabsf(m[1][2] * z) + fabsf(m[1][3]);
    float za = fabsf(m[2][0] * x) + fabsf(m[2][1] * y) + fabsf(m[2][2] * z) + fabsf(m[2][3]);
    V3 oerr = gamma(3.0f) * v3(xa, ya, za);
    V3 o = v3(xp, yp, zp);
    if (wp != 1.0f) o = o / wp;
    V3 dw = v3(m[0][0] * d.x + m[0][1] * d.y + m[0][2] * d.z, m[1][0] * d.x + m[1][1] * d.y + m[1][2] * d.z,
               m[2][0] * d.x + m[2][1] * d.y + m[2][2] * d.z);
    Ray r;
    r.t_max = INFINITY;
    float ls = length_squared(dw);
    if (ls > 0.0f) {
        float dt = dot(vabs(dw), oerr) / ls;
        o = o + dw * dt;
        r.t_max = INFINITY - dt;
    }
    r.o = o;
    r.d = dw;
    r.time = (1.0f - tu) * 0.0f + tu * 1.0f;
    return r;
}

}  // namespace bg

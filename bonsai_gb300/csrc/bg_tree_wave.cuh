// bg_tree_wave.cuh - shading of a level of the Whitted / direct-lighting tree wavefront (the shade
// kernel template and its helpers), shared by bg_tree_wave.cu and the translation units that
// instantiate the shade variants (bg_tree_shade_w.cu: Whitted; bg_tree_shade_d.cu: direct
// lighting), which compile in parallel.
#pragma once
#include "bg_estimate.cuh"
#include "bg_film.cuh"
#include "bg_kernels.h"
#include "bg_texture.cuh"
#include "bg_traverse.cuh"
#include "bg_warp.cuh"

namespace bg {

enum : uint32_t { TW_SHADOW = 2, TW_EXT_HEAD = 3, TW_SH_HEAD = 4, TW_OVERFLOW = 5 };
constexpr uint32_t TW_DIM_SPEC = 8, TW_DIM_LIGHTS = 12;

BG_D void store_rd(float4* rd, uint32_t i, const RayDiff& d) {
    rd[4 * i + 0] = make_float4(d.rxo.x, d.rxo.y, d.rxo.z, 0.0f);
    rd[4 * i + 1] = make_float4(d.ryo.x, d.ryo.y, d.ryo.z, 0.0f);
    rd[4 * i + 2] = make_float4(d.rxd.x, d.rxd.y, d.rxd.z, 0.0f);
    rd[4 * i + 3] = make_float4(d.ryd.x, d.ryd.y, d.ryd.z, 0.0f);
}
BG_D RayDiff load_rd(const float4* rd, uint32_t i) {
    RayDiff d;
    d.rxo = f4xyz(rd[4 * i + 0]);
    d.ryo = f4xyz(rd[4 * i + 1]);
    d.rxd = f4xyz(rd[4 * i + 2]);
    d.ryd = f4xyz(rd[4 * i + 3]);
    return d;
}
BG_D void add_L(const TreeWave& tw, uint32_t slot, RGB c) {
    if (is_black(c)) return;
    atomicAdd(&tw.L[slot].x, c.r);
    atomicAdd(&tw.L[slot].y, c.g);
    atomicAdd(&tw.L[slot].z, c.b);
}

// Appends a shadow ray (warp-collective: every lane calls it, lanes without a ray pass has = false).
BG_D void push_shadow(const TreeWave& tw, bool has, const Ray& r, int skip, RGB c, uint32_t slot) {
    const uint32_t pos = warp_append(&tw.counters[TW_SHADOW], has);
    if (!has) return;
    if (pos >= tw.sh_cap) {
        atomicOr(&tw.counters[TW_OVERFLOW], 1u);
        return;
    }
    tw.sh_o[pos] = make_float4(r.o.x, r.o.y, r.o.z, r.t_max);
    tw.sh_d[pos] = make_float4(r.d.x, r.d.y, r.d.z, __int_as_float(skip));
    tw.sh_c[pos] = make_float4(c.r, c.g, c.b, __uint_as_float(slot));
}

// estimate_direct (src/base/integrator.rs:330-437, PBRT) for one light as up to two shadow rays:
// the light sample's visibility ray and the BSDF sample's occlusion ray up to the light.  Both
// contributions are scaled by `scale` (beta / light-selection pdf).  Warp-collective.
BG_D void direct_rays(const Scene& sc, const TreeWave& tw, bool valid, const Isect& it, const BSDF& bsdf,
                      uint32_t light_prim, float us0, float us1, float ul0, float ul1, RGB scale, uint32_t slot) {
    const uint8_t flags = BSDF_ALL & ~BSDF_SPECULAR;
    bool h0 = false, h1 = false;
    Ray r0, r1;
    RGB c0 = rgb(0.0f), c1 = rgb(0.0f);
    if (valid) {
        LightSample ls = light_sample_any<false>(sc, light_prim, it, ul0, ul1);
        float scattering_pdf = 0.0f;
        if (ls.pdf > 0.0f && !is_black(ls.radiance)) {
            RGB f = bsdf.f<false>(it.wo, ls.wi, flags) * abs_dot(ls.wi, it.ns);
            scattering_pdf = bsdf.pdf<false>(it.wo, ls.wi, flags);
            if (!is_black(f)) {
                float w = power_heuristic(1.0f, ls.pdf, 1.0f, scattering_pdf);
                c0 = scale * (f * ls.radiance * w / ls.pdf);
                r0 = spawn_ray_to(it.p, it.p_err, it.n, it.time, ls.pt.p, ls.pt.p_err, ls.pt.n);
                h0 = true;
            }
        }
        BxSample bs = bsdf.sample<false>(it.wo, us0, us1, flags);
        RGB f = bs.f * abs_dot(bs.wi, it.ns);
        if (!is_black(f) && bs.pdf > 0.0f) {
            float t_light = 0.0f;
            V3 ln;
            float lpdf = light_pdf_any<false>(sc, light_prim, it, bs.wi, &t_light, &ln);
            if (lpdf != 0.0f) {
                float w = power_heuristic(1.0f, bs.pdf, 1.0f, lpdf);
                RGB li = light_radiance_along(sc, light_prim, bs.wi, ln);
                if (!is_black(li)) {
                    c1 = scale * (f * li * w / bs.pdf);
                    r1 = spawn_ray(it.p, it.p_err, it.n, it.time, bs.wi, false);
                    r1.t_max = t_light;
                    h1 = true;
                }
            }
        }
    }
    push_shadow(tw, h0, r0, -1, c0, slot);
    push_shadow(tw, h1, r1, light_prim == LIGHT_INFINITE ? -1 : (int)light_prim, c1, slot);
}

// Shades level d: emission, light sampling (kind 1 Whitted, 2 all lights, 3 one light) and the
// specular children of level d + 1 (PBRT mode: the dielectric as SpecularReflection +
// SpecularTransmission).
// Compiled for 6 resident CTAs per SM (at most 80 registers): production 1080p, 64 spp, Whitted
// 72.6 and direct lighting 36.8 Msamples/s, against 71.7 / 33.7 with 4 CTAs, 72.0 / 35.0 with 5
// and 67.2 / 30.6 unconstrained (196 registers).
#ifndef BG_TREE_SHADE_MINBLOCKS
#define BG_TREE_SHADE_MINBLOCKS 6
#endif
// KIND: 1 Whitted, 2 direct lighting with UniformSampleAll, 3 with UniformSampleOne (each variant
// carries only its own light-sampling code).
template <bool TEX, int KIND>
__global__ void __launch_bounds__(128, BG_TREE_SHADE_MINBLOCKS) k_tw_shade(Scene sc, RenderParams rp, TreeWave tw, uint32_t d,
                                                  uint64_t item0, uint32_t* err) {
    const uint32_t b = d & 1u, nb = b ^ 1u;
    const uint32_t n = min(tw.counters[b], tw.cap);
    const uint64_t npix = (uint64_t)rp.width * rp.height;
    const bool deeper = d + 1 < rp.max_depth;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < n; base += stride) {
        const uint32_t i = base + lane_id();
        bool valid = i < n;
        uint4 meta = make_uint4(0, 1, 0, 0);
        RGB beta = rgb(0.0f);
        Isect it;
        Ray ray;
        int prim = -1;
        if (valid) {
            meta = tw.meta[b][i];
            const float4 b4 = tw.beta[b][i];
            beta = rgb(b4.x, b4.y, b4.z);
            ray = load_ray(tw.ray_o[b][i], tw.ray_d[b][i]);
            prim = tw.hit[i].x;
            // background radiance of an escaped ray (whitted.rs:45-51, direct.rs:75-81)
            if (prim < 0 && sc.inf) add_L(tw, meta.x, beta * inf_radiance(sc, ray.d));
            valid = prim >= 0 && prim_isect(sc, prim, ray, &it);
        }
        const uint32_t slot = meta.x, node = meta.y;
        const uint64_t item = item0 + slot;
        const uint32_t pix = pixel_of((uint32_t)(item % npix), rp.width, rp.height, rp.pixel_tiles);
        const uint32_t s = rp.first_sample + (uint32_t)(item / npix);
        const Rng rng{pix, s, rp.seed, node - 1u};
        TexPoint tp;
        bool have_tp = false;
        RayDiff rd;
        const bool has_rd = TEX && valid && meta.w != 0u;
        BSDF bsdf;
        bsdf.n = 0;
        if (valid) {
            if (TEX) {
                if (has_rd) rd = load_rd(tw.rd[b], i);
                Isect tmp;
                if (!prim_isect(sc, prim, ray, &tmp, &tp.g)) tp.g = SurfaceGeom{};
                tp.p = it.p;
                tp.n = it.n;
                tp.d = compute_differentials(it.p, it.n, tp.g, has_rd ? &rd : nullptr);
                have_tp = true;
            }
            bsdf = make_bsdf<-1, false>(sc, it, have_tp ? &tp : nullptr, false);
            add_L(tw, slot, beta * emitted_radiance(sc, it, it.wo));
        }
        // light sampling: loops with the same trip count on every lane (warp-collective appends)
        if (sc.nlights > 0) {
            if constexpr (KIND == 1) {  // whitted.rs:176-192
                for (uint32_t j = 0; j < sc.nlights; ++j) {
                    bool has = false;
                    Ray sr;
                    RGB c = rgb(0.0f);
                    if (valid) {
                        LightSample ls = light_sample_any<false>(sc, sc.light_prims[j], it, rng.u(TW_DIM_LIGHTS + 2 * j),
                                                             rng.u(TW_DIM_LIGHTS + 2 * j + 1));
                        if (!is_black(ls.radiance) && ls.pdf != 0.0f) {
                            RGB f = bsdf.f<false>(it.wo, ls.wi, BSDF_ALL);
                            if (!is_black(f)) {
                                c = beta * (f * ls.radiance * abs_dot(ls.wi, it.ns) / ls.pdf);
                                sr = spawn_ray_to(it.p, it.p_err, it.n, it.time, ls.pt.p, ls.pt.p_err, ls.pt.n);
                                has = true;
                            }
                        }
                    }
                    push_shadow(tw, has, sr, -1, c, slot);
                }
            } else if constexpr (KIND == 2) {  // uniform_sample_all_lights (integrator.rs:274-307)
                for (uint32_t j = 0; j < sc.nlights; ++j) {
                    float u[4];
                    rng.block(TW_DIM_LIGHTS + 4 * j, u);
                    direct_rays(sc, tw, valid, it, bsdf, sc.light_prims[j], u[2], u[3], u[0], u[1], beta / 1.0f, slot);
                }
            } else {  // uniform_sample_one_light (integrator.rs:309-328)
                float u[8];
                rng.block(TW_DIM_LIGHTS, u);
                rng.block(TW_DIM_LIGHTS + 4, u + 4);
                const float count = (float)sc.nlights;
                const uint32_t li = (uint32_t)rmin(u[0] * count, count - 1.0f);
                direct_rays(sc, tw, valid, it, bsdf, sc.light_prims[li], u[3], u[4], u[1], u[2], beta / (1.0f / count),
                            slot);
            }
        }
        // specular children (specular_reflect / specular_transmit, integrator.rs:143-272)
        for (int k = 0; k < 2; ++k) {
            bool has = false;
            BxSample bs;
            if (valid && deeper) {
                float us[4];
                rng.block(TW_DIM_SPEC, us);
                const uint8_t type = k == 0 ? (BSDF_REFLECTION | BSDF_SPECULAR) : (BSDF_TRANSMISSION | BSDF_SPECULAR);
                bs = bsdf.sample<false>(it.wo, us[2 * k], us[2 * k + 1], type);
                has = bs.pdf > 0.0f && !is_black(bs.f) && abs_dot(bs.wi, it.ns) != 0.0f;
            }
            const uint32_t pos = warp_append(&tw.counters[nb], has);
            if (!has) continue;
            if (pos >= tw.cap) {
                atomicOr(&tw.counters[TW_OVERFLOW], 1u);
                continue;
            }
            const Ray c = spawn_ray(it.p, it.p_err, it.n, it.time, bs.wi, false);
            const RGB cb = beta * (bs.f * abs_dot(bs.wi, it.ns) / bs.pdf);
            tw.ray_o[nb][pos] = make_float4(c.o.x, c.o.y, c.o.z, c.t_max);
            tw.ray_d[nb][pos] = make_float4(c.d.x, c.d.y, c.d.z, c.time);
            tw.beta[nb][pos] = make_float4(cb.r, cb.g, cb.b, 0.0f);
            const bool crd = TEX && has_rd && have_tp;
            tw.meta[nb][pos] = make_uint4(slot, 2u * node + (uint32_t)k, d + 1, crd ? 1u : 0u);
            if (crd) store_rd(tw.rd[nb], pos, specular_diff(it, tp, rd, bs.wi, bsdf.eta, k == 1));
        }
    }
}

// Launches the shade kernel of level d for integrator `kind` (bg_tree_shade_w.cu, bg_tree_shade_d.cu).
void launch_tw_shade_whitted(const Scene& sc, const RenderParams& rp, const TreeWave& tw, uint32_t d, uint64_t item0,
                             uint32_t* err, dim3 grid, dim3 block, cudaStream_t s);
void launch_tw_shade_direct(int kind, const Scene& sc, const RenderParams& rp, const TreeWave& tw, uint32_t d,
                            uint64_t item0, uint32_t* err, dim3 grid, dim3 block, cudaStream_t s);

}  // namespace bg

// bg_estimate.cuh - per-thread ray queries over any BVH layout and estimate_direct for the
// per-sample megakernels (the reference-layout path integrator, Whitted, direct lighting).
#pragma once
#include "bg_shading.cuh"
#include "bg_traverse.cuh"

namespace bg {

// One ray against the scene: LAYOUT 1 = reference binary layout, 2 = 2-wide, 8 = 8-wide.
// Closest hit: returns the prim and leaves the hit distance in ray.t_max; ANY: any hit before
// ray.t_max.
template <int LAYOUT, bool ANY>
BG_D int trace_one(const Scene& sc, Ray& ray, uint32_t* err) {
    if constexpr (LAYOUT == 1) return ref_traverse<ANY>(sc, ray, err, nullptr);
    else if constexpr (LAYOUT == 2) return bvh2_traverse<ANY>(sc, ray, err);
    else return bvh8_traverse<ANY>(sc, ray, err);
}

// estimate_direct (src/base/integrator.rs:330-437) for a per-thread integrator, its shadow and
// BSDF-sampled rays traced by trace_one over the scene's layout.
template <bool REF, int LAYOUT>
BG_D RGB estimate_direct_mk(const Scene& sc, const Isect& it, const BSDF& bsdf, uint32_t light_prim, float us0,
                             float us1, float ul0, float ul1, uint32_t* err) {
    const uint8_t flags = BSDF_ALL & ~BSDF_SPECULAR;
    RGB out = rgb(0.0f);
    LightSample ls = light_sample_any<REF>(sc, light_prim, it, ul0, ul1);
    float scattering_pdf = 0.0f;
    if (ls.pdf > 0.0f && !is_black(ls.radiance)) {
        RGB f = bsdf.f<REF>(it.wo, ls.wi, flags) * abs_dot(ls.wi, it.ns);
        scattering_pdf = bsdf.pdf<REF>(it.wo, ls.wi, flags);
        if (!is_black(f)) {
            Ray sr = spawn_ray_to(it.p, it.p_err, it.n, it.time, ls.pt.p, ls.pt.p_err, ls.pt.n);
            if (trace_one<LAYOUT, true>(sc, sr, err) >= 0) ls.radiance = rgb(0.0f);
            if (!is_black(ls.radiance)) {
                float w = power_heuristic(1.0f, ls.pdf, 1.0f, scattering_pdf);
                out = out + f * ls.radiance * w / ls.pdf;
            }
        }
    }
    BxSample bs = bsdf.sample<REF>(it.wo, us0, us1, flags);
    RGB f = bs.f * abs_dot(bs.wi, it.ns);
    bool sampled_specular = (bs.stype & BSDF_SPECULAR) != 0;
    // REF (F2): ray along the light sample's direction with the light half's pdf, any emitter
    V3 wdir = REF ? ls.wi : bs.wi;
    float spdf = REF ? scattering_pdf : bs.pdf;
    if (!is_black(f) && spdf > 0.0f) {
        float w = 1.0f;
        if (!sampled_specular) {
            float lpdf = light_pdf_any<REF>(sc, light_prim, it, wdir, nullptr);
            if (lpdf == 0.0f) return out;
            w = power_heuristic(1.0f, spdf, 1.0f, lpdf);
        }
        Ray ray = spawn_ray(it.p, it.p_err, it.n, it.time, wdir, REF);
        Ray rr = ray;
        int prim = trace_one<LAYOUT, false>(sc, rr, err);
        RGB li = rgb(0.0f);
        if (prim < 0) {
            // an escaping ray sees Light::radiance: the environment map of an infinite light
            if (light_prim == LIGHT_INFINITE) li = inf_radiance(sc, wdir);
        } else if (REF ? prim_emission(sc, prim) >= 0 : prim == (int)light_prim) {
            Isect lit;
            if (prim_isect(sc, prim, ray, &lit)) li = emitted_radiance(sc, lit, -wdir);
        }
        if (!is_black(li)) out = out + f * li * w / spdf;
    }
    return out;
}

// PathIntegrator::radiance (src/integrators/path.rs:51-146) over the reference BVH.

}  // namespace bg

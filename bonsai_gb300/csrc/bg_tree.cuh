// bg_tree.cuh - the Whitted and direct-lighting integrators (src/integrators/whitted.rs,
// src/integrators/direct.rs) on the device.
//
// Both are SamplerIntegrators whose radiance recursion branches only at specular surfaces
// (specular_reflect / specular_transmit, src/base/integrator.rs:143-272): every camera sample is
// one camera ray, its light-sampling rays and - at a dielectric split into SpecularReflection +
// SpecularTransmission - a binary tree of specular rays at most max_depth deep.  One thread runs a
// sample's whole tree depth-first with an explicit stack of pending specular rays (at most one per
// level), tracing every ray with the per-thread traversal of the scene's BVH layout.  A sample's
// contributions are summed in registers and reach the film once, through the sanity checks of
// SamplerIntegrator::render.
//
// Random numbers: the counter RNG keyed by (pixel, sample) with stream = node id - 1 of the tree
// (root 1, reflected child 2k, transmitted child 2k + 1).  Dimensions per node: camera 0-4 (root),
// specular reflection 8-9, specular transmission 10-11, light sampling from 12 (Whitted: light j at
// 12 + 2j; direct, all lights: light j at 12 + 4j (u_light, then u_scattering); direct, one light:
// pick 12, u_light 13-14, u_scattering 15-16).  The reference draws the same quantities from one
// sequential sampler stream, so parity with it is statistical.
#pragma once
#include "bg_estimate.cuh"
#include "bg_film.cuh"
#include "bg_kernels.h"
#include "bg_texture.cuh"

namespace bg {

constexpr uint32_t DIM_SPEC = 8, DIM_LIGHTS = 12;

struct TreeRay {
    Ray ray;
    RayDiff rd;
    RGB beta;
    uint32_t depth, node;
    bool has_rd;
};

// kind: 1 Whitted, 2 direct lighting with UniformSampleAll, 3 direct lighting with UniformSampleOne
// (a launch-uniform branch).
template <bool REF, int LAYOUT>
BG_D RGB tree_radiance(const Scene& sc, const RenderParams& rp, int kind, Ray cam_ray, const RayDiff* cam_rd,
                       uint32_t pix, uint32_t s, uint32_t* err) {
    TreeRay st[TREE_STACK];
    int sp = 0;
    st[sp].ray = cam_ray;
    st[sp].has_rd = cam_rd != nullptr;
    if (cam_rd) st[sp].rd = *cam_rd;
    st[sp].beta = rgb(1.0f);
    st[sp].depth = 0;
    st[sp].node = 1;
    ++sp;
    RGB L = rgb(0.0f);
    while (sp > 0) {
        const TreeRay nd = st[--sp];
        Ray r = nd.ray;
        const int prim = trace_one<LAYOUT, false>(sc, r, err);
        if (prim < 0) {  // background radiance (whitted.rs:45-51, direct.rs:75-81); area lights add none
            if (sc.inf) L = L + nd.beta * inf_radiance(sc, nd.ray.d);
            continue;
        }
        Isect it;
        if (!prim_isect(sc, prim, nd.ray, &it)) continue;
        const Rng rng{pix, s, rp.seed, nd.node - 1u};
        // texture inputs: every hit of a textured scene whose ray has differentials carries them,
        // since the specular children's differentials derive from them
        TexPoint tp;
        bool have_tp = false;
        if (sc.ntex) {
            Isect tmp;
            if (!prim_isect(sc, prim, nd.ray, &tmp, &tp.g)) tp.g = SurfaceGeom{};
            tp.p = it.p;
            tp.n = it.n;
            tp.d = compute_differentials(it.p, it.n, tp.g, nd.has_rd ? &nd.rd : nullptr);
            have_tp = true;
        }
        const BSDF bsdf = make_bsdf<-1, REF>(sc, it, have_tp ? &tp : nullptr, false);
        L = L + nd.beta * emitted_radiance(sc, it, it.wo);
        if (sc.nlights > 0) {
            if (kind == 1) {  // whitted.rs:176-192
                for (uint32_t j = 0; j < sc.nlights; ++j) {
                    const uint32_t lp = sc.light_prims[j];
                    LightSample ls = light_sample_any<REF>(sc, lp, it, rng.u(DIM_LIGHTS + 2 * j), rng.u(DIM_LIGHTS + 2 * j + 1));
                    if (is_black(ls.radiance) || ls.pdf == 0.0f) continue;
                    RGB f = bsdf.f<REF>(it.wo, ls.wi, BSDF_ALL);
                    if (is_black(f)) continue;
                    Ray sr = spawn_ray_to(it.p, it.p_err, it.n, it.time, ls.pt.p, ls.pt.p_err, ls.pt.n);
                    if (trace_one<LAYOUT, true>(sc, sr, err) >= 0) continue;
                    L = L + nd.beta * (f * ls.radiance * abs_dot(ls.wi, it.ns) / ls.pdf);
                }
            } else if (kind == 2) {  // uniform_sample_all_lights (integrator.rs:274-307)
                for (uint32_t j = 0; j < sc.nlights; ++j) {
                    float u[4];
                    rng.block(DIM_LIGHTS + 4 * j, u);
                    RGB ld = estimate_direct_mk<REF, LAYOUT>(sc, it, bsdf, sc.light_prims[j], u[2], u[3], u[0], u[1], err);
                    L = L + nd.beta * (ld / 1.0f);  // one sample per DiffuseAreaLight (light.rs:51-53)
                }
            } else {  // uniform_sample_one_light (integrator.rs:309-328)
                float u[8];
                rng.block(DIM_LIGHTS, u);
                rng.block(DIM_LIGHTS + 4, u + 4);
                const float count = (float)sc.nlights;
                const uint32_t li = (uint32_t)rmin(u[0] * count, count - 1.0f);
                RGB ld = estimate_direct_mk<REF, LAYOUT>(sc, it, bsdf, sc.light_prims[li], u[3], u[4], u[1], u[2], err);
                L = L + nd.beta * (ld / (1.0f / count));
            }
        }
        if (nd.depth + 1 < rp.max_depth) {
            float us[4];
            rng.block(DIM_SPEC, us);
            // pushed transmission first so the reflected subtree is walked first, as the reference
            for (int k = 1; k >= 0; --k) {
                const uint8_t type = k == 0 ? (BSDF_REFLECTION | BSDF_SPECULAR) : (BSDF_TRANSMISSION | BSDF_SPECULAR);
                BxSample bs = bsdf.sample<REF>(it.wo, us[2 * k], us[2 * k + 1], type);
                if (!(bs.pdf > 0.0f) || is_black(bs.f) || abs_dot(bs.wi, it.ns) == 0.0f) continue;
                if (sp >= TREE_STACK) {
                    atomicOr(err, ERR_STACK_OVERFLOW);
                    continue;
                }
                TreeRay& c = st[sp++];
                c.ray = spawn_ray(it.p, it.p_err, it.n, it.time, bs.wi, REF);
                c.has_rd = nd.has_rd && have_tp;
                if (c.has_rd) c.rd = specular_diff(it, tp, nd.rd, bs.wi, bsdf.eta, k == 1);
                c.beta = nd.beta * (bs.f * abs_dot(bs.wi, it.ns) / bs.pdf);
                c.depth = nd.depth + 1;
                c.node = 2u * nd.node + (uint32_t)k;
            }
        }
    }
    return L;
}

template <bool REF, int LAYOUT>
__global__ void __launch_bounds__(128) k_tree(Scene sc, Camera cam, RenderParams rp, FilmBuffers film, int kind,
                                              uint32_t* err) {
    const uint64_t npix = (uint64_t)rp.width * rp.height;
    const uint64_t total = npix * rp.spp;
    for (uint64_t item = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; item < total;
         item += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t pix = (uint32_t)(item % npix);
        const uint32_t s = rp.first_sample + (uint32_t)(item / npix);
        const Rng rng{pix, s, rp.seed, 0u};
        const CameraUs cu = camera_us(rp.strat, REF, rng, cam.lens_radius > 0.0f);  // sampled_dimensions <= 1: camera only
        const float fx = (float)(pix % rp.width) + cu.fx, fy = (float)(pix / rp.width) + cu.fy;
        const Ray ray = camera_ray(cam, fx, fy, cu.time, cu.lx, cu.ly);
        RayDiff rd;
        if (sc.ntex) rd = camera_diff(cam, fx, fy, ray, rp.diff_scale, cu.lx, cu.ly);
        RGB L = tree_radiance<REF, LAYOUT>(sc, rp, kind, ray, sc.ntex ? &rd : nullptr, pix, s, err);
        film_add(film, pix, L);
    }
}

// Launches k_tree<false, 1> (PBRT mode; bg_integrators_pbrt.cu, compiled in parallel).
void launch_tree_pbrt(int kind, const Scene& sc, const Camera& cam, const RenderParams& rp, const FilmBuffers& film,
                      uint32_t* err, dim3 grid, dim3 block, cudaStream_t s);

}  // namespace bg

// bg_wave.cuh - device code shared by the wavefront translation units: the path state word,
// camera-ray generation, texture inputs of a path vertex, guiding records, next-event estimation
// and continuation of a vertex (scatter_vertex) and the shade kernel template.
// The shade kernels are instantiated in bg_shade_plain.cu (single-scene renders) and
// bg_shade_aux.cu (guided and batch renders) so that their compilation runs in parallel.
#pragma once
#include "bg_guide.cuh"
#include "bg_guide_kernels.h"
#include "bg_kernels.h"
#include "bg_shading.cuh"
#include "bg_traverse.cuh"
#include "bg_film.cuh"
#include "bg_estimate.cuh"
#include "bg_warp.cuh"

namespace bg {

// ================================================================ textures
// Texture inputs at a hit whose material is textured (nullptr otherwise): the surface geometry
// re-derived from the hit and the screen-space differentials of ray differentials `rd`.
BG_D const TexPoint* tex_point(const Scene& sc, const Isect& it, const Ray& ray, const RayDiff* rd, TexPoint* tp) {
    if (!sc.ntex || !material_textured(sc.mats[prim_material(sc, it.prim)])) return nullptr;
    Isect tmp;
    if (!prim_isect(sc, it.prim, ray, &tmp, &tp->g)) tp->g = SurfaceGeom{};
    tp->p = it.p;
    tp->n = it.n;
    tp->d = compute_differentials(it.p, it.n, tp->g, rd);
    return tp;
}
// The camera ray differentials of path (pixel, sample) at its camera sample's film position (the
// same sampler values as the ray's generation); `cam_ray` is its camera ray.
BG_D RayDiff path_camera_diff(const RenderParams& rp, uint32_t pix, uint32_t s, const Ray& cam_ray) {
    const CameraUs cu = camera_us(rp.strat, false, Rng{pix, s, rp.seed}, rp.cam.lens_radius > 0.0f, false);
    const float fx = (float)(pix % rp.width) + cu.fx, fy = (float)(pix / rp.width) + cu.fy;
    return camera_diff(rp.cam, fx, fy, cam_ray, rp.diff_scale, cu.lx, cu.ly);
}
// BSDF of a path vertex: textured materials read the camera differentials at the first hit
// (PathIntegrator spawns later rays without differentials, path.rs:139).
// TEX: texture support compiled in (it costs the shade kernels about 30 registers).
template <int CLS, bool TEX>
BG_D BSDF path_bsdf(const Scene& sc, const RenderParams& rp, uint32_t pix, uint32_t s, uint32_t bounce, const Ray& ray,
                    const Isect& it) {
    if (!TEX || !sc.ntex) return make_bsdf<CLS>(sc, it);
    TexPoint tp;
    RayDiff rd;
    if (bounce == 0) rd = path_camera_diff(rp, pix, s, ray);
    return make_bsdf<CLS>(sc, it, tex_point(sc, it, ray, bounce == 0 ? &rd : nullptr, &tp));
}

// ================================================================ wavefront (PBRT)
// Path state word: bits 0-7 bounce, 8 specular bounce, 9 pending NEE contribution, 10 open
// training record, 11 pending light-sample record, 12-15 training records written, 16-23 / 24-31 the sampler's get_1d / get_2d
// calls so far (saturating at 255; calls below sampled_dimensions take stratified values).
enum : uint32_t { ST_SPECULAR = 1u << 8, ST_PENDING = 1u << 9, ST_REC_OPEN = 1u << 10, ST_LREC = 1u << 11 };
constexpr uint32_t ST_REC_SHIFT = 12, ST_REC_MASK = 0xFu << ST_REC_SHIFT;
BG_D uint32_t st_k1(uint32_t st) { return (st >> 16) & 0xFFu; }
BG_D uint32_t st_k2(uint32_t st) { return st >> 24; }
BG_D uint32_t st_set_k(uint32_t st, uint32_t k1, uint32_t k2) {
    return (st & 0xFFFFu) | (min(k1, 255u) << 16) | (min(k2, 255u) << 24);
}
enum : uint32_t { C_Q0 = 0, C_Q1 = 1, C_SHADOW = 2, C_DONE = 3, C_EXT_HEAD = 4, C_SH_HEAD = 5, C_CLS = 6 };
constexpr int NCLS = 5;          // material classes 0..3 (bg_material_type) + misses
constexpr int CLS_MISS = 4;

// Camera ray of (pixel, sample) into path slot i (PerspectiveCamera::generate_ray).
BG_D void generate_one(const Camera& cam, const RenderParams& rp, const WaveBuffers& wb, uint32_t i, uint32_t pix,
                       uint32_t s) {
    Rng rng{pix, s, rp.seed};
    const CameraUs cu = camera_us(rp.strat, false, rng, cam.lens_radius > 0.0f);
    float fx = (float)(pix % rp.width) + cu.fx, fy = (float)(pix / rp.width) + cu.fy;
    Ray r = camera_ray(cam, fx, fy, cu.time, cu.lx, cu.ly);
    wb.ray_o[i] = make_float4(r.o.x, r.o.y, r.o.z, r.t_max);
    wb.ray_d[i] = make_float4(r.d.x, r.d.y, r.d.z, r.time);
    wb.pixel[i] = pix;
    wb.sample[i] = s;
    wb.state[i] = st_set_k(0u, 1u, 2u);  // the camera sample made one get_1d and two get_2d calls
    wb.beta[i] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    wb.L[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    wb.queue[0][i] = i;
}

BG_D void generate_paths(const Camera& cam, const RenderParams& rp, const WaveBuffers& wb, uint64_t item0,
                         uint32_t nitems, uint32_t first_sample) {
    const uint64_t npix = (uint64_t)rp.width * rp.height;
    if (blockIdx.x == 0 && threadIdx.x == 0) wb.counters[C_Q0] = nitems;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nitems; i += gridDim.x * blockDim.x) {
        uint64_t item = item0 + i;
        generate_one(cam, rp, wb, i, pixel_of((uint32_t)(item % npix), rp.width, rp.height, rp.pixel_tiles),
                     first_sample + (uint32_t)(item / npix));
    }
}

// The scene / render parameters / film of a path: the kernel's own in a single-scene render, the
// path's table entry in a batch render.
template <bool MULTI, class T>
BG_D const T& pick(const T& single, const T* multi) {
    if constexpr (MULTI) return *multi;
    else return single;
}

// Adds the pending next-event contribution of the previous vertex:
// L += beta_nee * ((part0 + part1) / light_pdf)  (path.rs:107-109, integrator.rs:327).
BG_D RGB apply_pending(const WaveBuffers& wb, uint32_t slot, RGB L, uint32_t state, uint32_t nlights) {
    if (!(state & ST_PENDING)) return L;
    float4 p0 = wb.pending[2 * slot], p1 = wb.pending[2 * slot + 1];
    RGB ld = rgb(0.0f);
    if (p0.w != 0.0f) ld = ld + rgb(p0.x, p0.y, p0.z);
    if (p1.w != 0.0f) ld = ld + rgb(p1.x, p1.y, p1.z);
    float4 nb = wb.nee_beta[slot];
    float light_pdf = 1.0f / (float)nlights;
    return L + rgb(nb.x, nb.y, nb.z) * (ld / light_pdf);
}

// ---- guiding: training records and network queries
BG_D float4* rec_ptr(const GuideWave& gw, uint32_t k, uint32_t f, uint32_t slot) {
    return gw.rec + ((size_t)(k * GUIDE_REC_F4 + f) * gw.cap + slot);
}
BG_D uint32_t rec_count(uint32_t state) { return (state & ST_REC_MASK) >> ST_REC_SHIFT; }

// Closes the open record at the vertex its direction reached.  `L_after` is the radiance the path
// holds once this vertex's emission is counted (if the estimator counts it here), `le_beta` that
// emission times the path throughput.  Everything the path adds after L_after arrived along the
// recorded direction indirectly (the indirect target); the emission found here, divided by the
// recording vertex's throughput, is the direct target f |cos| Le / p, stored in .w.
BG_D uint32_t close_record(const GuideWave& gw, const WaveBuffers& wb, uint32_t slot, uint32_t state, RGB L_after,
                           RGB le_beta) {
    if (!(state & ST_REC_OPEN) || slot >= gw.cap) return state;
    uint32_t k = rec_count(state) - 1;
    float w_direct = 0.0f;
    if (!is_black(le_beta)) {
        const float4 r3 = *rec_ptr(gw, k, 3, slot);
        w_direct = luminance(rgb(r3.y > 0.0f ? le_beta.r / r3.y : 0.0f, r3.z > 0.0f ? le_beta.g / r3.z : 0.0f,
                                 r3.w > 0.0f ? le_beta.b / r3.w : 0.0f));
    }
    *rec_ptr(gw, k, 4, slot) = make_float4(L_after.r, L_after.g, L_after.b, w_direct);
    return state & ~ST_REC_OPEN;
}

// The render's inference writes the mixture records of its three class ranges (gw.cap queries
// each) head-major: head 1's record of a query lies this many floats after head 0's.
BG_D size_t mix_head_stride(const GuideWave& gw) { return (size_t)3 * gw.cap * GUIDE_MIX_HEAD; }

struct GuideQuery {  // p_norm.xyz n.x | n.yz wo.xy | wo.z
    float4 a, b, c;
};
BG_D GuideQuery make_query(const GuideWave& gw, const Isect& it, V3 wo) {
    V3 pn = v3(rclamp((it.p.x - gw.bmin.x) * gw.binv.x, 0.0f, 1.0f), rclamp((it.p.y - gw.bmin.y) * gw.binv.y, 0.0f, 1.0f),
               rclamp((it.p.z - gw.bmin.z) * gw.binv.z, 0.0f, 1.0f));
    V3 n = face_forward(it.ns, wo);
    return {make_float4(pn.x, pn.y, pn.z, n.x), make_float4(n.y, n.z, wo.x, wo.y), make_float4(wo.z, 0.0f, 0.0f, 0.0f)};
}

// Opens a training record for a sampled continuation wi (p_b = BSDF pdf of wi, beta = throughput
// before the vertex).
BG_D uint32_t open_record(const GuideWave& gw, const WaveBuffers& wb, uint32_t slot, uint32_t state,
                          const GuideQuery& q, V3 wi, float p_b, RGB beta) {
    uint32_t k = rec_count(state);
    if (k >= (uint32_t)GUIDE_MAXREC || slot >= gw.cap) return state;
    *rec_ptr(gw, k, 0, slot) = q.a;
    *rec_ptr(gw, k, 1, slot) = q.b;
    *rec_ptr(gw, k, 2, slot) = make_float4(q.c.x, wi.x, wi.y, wi.z);
    *rec_ptr(gw, k, 3, slot) = make_float4(p_b, beta.r, beta.g, beta.b);
    return (state & ~ST_REC_MASK) | ((k + 1) << ST_REC_SHIFT) | ST_REC_OPEN;
}

// Integer hash in [0, 1) for choosing the paths that record training samples (not part of the
// estimator).
BG_D float hash_unit(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u ^ (c + 0x165667B1u) * 0xC2B2AE3Du;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return (float)(h >> 8) * 0x1p-24f;
}

// The light sample of a recording vertex as a training sample of the next-event head: the
// sampled direction with weight f |cos| Le / p_light (luminance; p_light includes the 1 / nlights
// light choice), stored until the shadow ray tells whether the light was seen (ST_LREC).
BG_D float4* lrec_ptr(const GuideWave& gw, uint32_t bounce, uint32_t slot) {
    return gw.lrec + 4 * ((size_t)(bounce & 1) * gw.cap + slot);
}
// Warp-collective: lanes with `emit` (a resolved, visible light sample of the vertex at `bounce`)
// append that sample to the pool.
BG_D void emit_light_record(const GuideWave& gw, uint32_t bounce, uint32_t slot, bool emit) {
    if (!__any_sync(FULL, emit)) return;
    const uint32_t pos = warp_append(&gw.ctr[1], emit);
    if (emit && pos < gw.pool_cap) {
        const float4* r = lrec_ptr(gw, bounce, slot);
        float4* o = gw.pool + (size_t)GUIDE_SAMPLE_F4 * pos;
        o[0] = r[0];
        o[1] = r[1];
        o[2] = r[2];
        o[3] = r[3];
    }
    const uint32_t tot = __popc(__ballot_sync(FULL, emit));
    if (lane_id() == 0) atomicAdd(&gw.ctr[0], tot);
}

// Turns the records of finished paths into training samples.  Warp-collective: every lane calls
// it, lanes without a finished path pass nrec = 0.  A lane first reads the closing halves of all
// its records (independent loads, in flight together) and marks the positive ones; the warp then
// reserves pool positions for all of them with one atomic and each lane copies its kept records.
BG_D void emit_records(const GuideWave& gw, const WaveBuffers& wb, uint32_t slot, uint32_t nrec, RGB L_end) {
    if (!__any_sync(FULL, nrec > 0)) return;
    float w[GUIDE_MAXREC], wd[GUIDE_MAXREC], pb[GUIDE_MAXREC];
    uint32_t keep = 0;
#pragma unroll
    for (int k = 0; k < GUIDE_MAXREC; ++k) {
        w[k] = wd[k] = pb[k] = 0.0f;
        if ((uint32_t)k < nrec) {
            const float4 r3 = *rec_ptr(gw, k, 3, slot);
            const float4 r4 = *rec_ptr(gw, k, 4, slot);
            RGB d = L_end - rgb(r4.x, r4.y, r4.z);
            // (L_end - L_after) / beta = f |cos| Li_indirect / p of the recorded direction (head 0);
            // r4.w = f |cos| Le / p, the emission the direction reached (head 1)
            RGB li = rgb(r3.y > 0.0f ? d.r / r3.y : 0.0f, r3.z > 0.0f ? d.g / r3.z : 0.0f,
                         r3.w > 0.0f ? d.b / r3.w : 0.0f);
            float wi = fmaxf(luminance(li), 0.0f);
            w[k] = isfinite(wi) ? wi : 0.0f;
            wd[k] = r4.w > 0.0f && isfinite(r4.w) ? r4.w : 0.0f;
            pb[k] = r3.x;
            // every positive record of a path chosen for the pool (when it opened its records) is kept
            if (w[k] > 0.0f || wd[k] > 0.0f) keep |= 1u << k;
        }
    }
    const uint32_t n = __popc(keep), lane = lane_id();
    uint32_t incl = n;  // inclusive prefix sum over the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(FULL, incl, o);
        if (lane >= (uint32_t)o) incl += t;
    }
    const uint32_t total = __shfl_sync(FULL, incl, 31);
    if (total == 0) return;
    uint32_t base = 0;
    if (lane == 31) {
        base = atomicAdd(&gw.ctr[1], total);
        atomicAdd(&gw.ctr[0], total);
    }
    uint32_t pos = __shfl_sync(FULL, base, 31) + incl - n;
#pragma unroll
    for (int k = 0; k < GUIDE_MAXREC; ++k) {
        if (!((keep >> k) & 1u)) continue;
        if (pos < gw.pool_cap) {
            float4* o = gw.pool + (size_t)GUIDE_SAMPLE_F4 * pos;
            o[0] = *rec_ptr(gw, k, 0, slot);
            o[1] = *rec_ptr(gw, k, 1, slot);
            o[2] = *rec_ptr(gw, k, 2, slot);
            o[3] = make_float4(pb[k], w[k], wd[k], 0.0f);
        }
        ++pos;
    }
}

// Everything a non-specular or specular vertex does after its emission: next-event estimation
// (uniform_sample_one_light + estimate_direct, src/base/integrator.rs:309-437, the occlusion tests
// deferred to k_shadow), the BSDF-sampled continuation (src/integrators/path.rs:110-143) and
// Russian roulette.  `mix` (guided vertices, the query's two mixtures) replaces the BSDF by the
// one-sample mixture c * guide + (1 - c) * BSDF of head 1 in estimate_direct's second strategy
// (GW_NEE; the direction is drawn from it and both MIS weights use its pdf) and by that of head 0
// for the continuation (GW_CONT; the throughput divides by its pdf), so the estimator stays
// unbiased whatever the network outputs.
struct VertexOut {
    bool cont = false, finished = false;
    bool push_sh[2] = {false, false};
    float4 sh_o[2], sh_d[2];
};

// The stratified values a bounce may take (get_1d calls k1 and k1 + 1, get_2d calls k2 .. k2 + 2:
// with light sampling the bounce makes 1D k1, 2D k2, k2 + 1, the BSDF's 2D k2 + 2 and the roulette's
// 1D k1 + 1; without, the BSDF's 2D k2 and the roulette's 1D k1), -1 where the call falls through to
// the counter RNG.  A shade thread computes them when it picks up a path, where few registers are
// live, into its column of shared memory (8 rows, stride SU_STRIDE).
constexpr uint32_t SU_STRIDE = 128;
// Not inlined: renders with the independent sampler never call it, and its code (permutations, cycle
// walking) would otherwise sit among the shade kernels' hot instructions.
static __device__ __noinline__ void strat_prefetch(const StratParams& sp, uint32_t pix, uint32_t sample, uint64_t seed, uint32_t k1,
                         uint32_t k2, float* col) {
    col[0] = k1 < sp.dims ? strat_1d(sp, false, pix, sample, seed, k1) : -1.0f;
    col[SU_STRIDE] = k1 + 1 < sp.dims ? strat_1d(sp, false, pix, sample, seed, k1 + 1) : -1.0f;
    for (uint32_t j = 0; j < 3; ++j) {
        const float2 v = k2 + j < sp.dims ? strat_2d(sp, false, pix, sample, seed, k2 + j) : make_float2(-1.0f, -1.0f);
        col[(2 + 2 * j) * SU_STRIDE] = v.x;
        col[(3 + 2 * j) * SU_STRIDE] = v.y;
    }
}
BG_D void strat_apply(const float* su, bool nee, float u[8]) {
    const float a = su[0], b = su[SU_STRIDE];
    auto pair = [&](int row, int slot) {
        const float x = su[row * SU_STRIDE];
        if (x >= 0.0f) {
            u[slot] = x;
            u[slot + 1] = su[(row + 1) * SU_STRIDE];
        }
    };
    if (nee) {
        if (a >= 0.0f) u[BD_LIGHT] = a;
        pair(2, BD_ULIGHT);
        pair(4, BD_USCAT);
        pair(6, BD_BSDF);
        if (b >= 0.0f) u[BD_RR] = b;
    } else {
        pair(2, BD_BSDF);
        if (a >= 0.0f) u[BD_RR] = a;
    }
}

// INF: the scene's light list may hold more than triangles - the infinite light, emitting spheres
// or quadrics (variants launched only for such scenes, general_lights, so that the others carry
// none of that code).
// SHL: emitting spheres / quadrics may be in the light list (with INF).
template <int CLS, bool TEX = false, bool INF = false, bool SHL = INF>
BG_D void scatter_vertex(const Scene& sc, const RenderParams& rp, const WaveBuffers& wb, const GuideWave& gw,
                         uint32_t slot, uint32_t bounce, const Ray& ray, const Isect& it, RGB& beta, float& eta_scale,
                         uint32_t& state, const MixView* mix, const float* ug, bool record, VertexOut& out,
                         const float* su = nullptr) {
    constexpr bool GUIDABLE = CLS >= 0 && CLS <= 2;
    Rng rng{wb.pixel[slot], wb.sample[slot], rp.seed};
    const uint32_t ub = DIM_BOUNCE0 + DIMS_PER_BOUNCE * bounce;
    float u[8];
    rng.block(ub, u);
    rng.block(ub + 4, u + 4);
    BSDF bsdf = path_bsdf<CLS, TEX>(sc, rp, wb.pixel[slot], wb.sample[slot], bounce, ray, it);
    const bool nee = bsdf.num_components(BSDF_ALL & ~BSDF_SPECULAR) > 0 && sc.nlights > 0;
    // the bounce's sampler calls: [get_1d light, get_2d u_light, get_2d u_scattering,] get_2d BSDF,
    // get_1d roulette (made only when the roulette test runs; its value is drawn here regardless)
    if (su) strat_apply(su, nee, u);  // the stratified sampler's values, prefetched by the shade thread
    // the counters move past this bounce's calls now (the roulette's get_1d when its test runs)
    state = st_set_k(state, st_k1(state) + (nee ? 1u : 0u), st_k2(state) + (nee ? 3u : 1u));
    // paths chosen for the training pool (a per-path choice with probability keep_prob, so the
    // other paths write nothing) record every sampled continuation and light sample
    const bool chosen = GUIDABLE && record && hash_unit(wb.pixel[slot], wb.sample[slot], 0x5EEDu) < gw.keep_prob;
    GuideQuery gq;
    if (chosen) gq = make_query(gw, it, -ray.d);
    // `mix` is the query's two-head record: head 0 (at mix) for the continuation (GW_CONT), head 1
    // for estimate_direct's second strategy (GW_NEE)
    const MixView nview{mix ? mix->m + mix_head_stride(gw) : nullptr};
    const MixView* nmix = GUIDABLE && mix && (gw.flags & GW_NEE) ? &nview : nullptr;
    if (nee) {
        const uint8_t flags = BSDF_ALL & ~BSDF_SPECULAR;
        float count = (float)sc.nlights;
        uint32_t light_prim = sc.light_prims[(uint32_t)rmin(u[BD_LIGHT] * count, count - 1.0f)];
        float4 pend[2] = {make_float4(0, 0, 0, 0), make_float4(0, 0, 0, 0)};
        // pdf of the second strategy for a direction
        auto strategy_pdf = [&](V3 w) {
            float pb = bsdf.pdf<false>(it.wo, w, flags);
            if (!nmix) return pb;
            const float c = nmix->c();
            return c * nmix->pdf(w) + (1.0f - c) * pb;
        };
        LightSample ls = INF ? light_sample_any<false, SHL>(sc, light_prim, it, u[BD_ULIGHT], u[BD_ULIGHT + 1])
                             : light_sample<false, false>(sc, light_prim, it, u[BD_ULIGHT], u[BD_ULIGHT + 1]);
        if (ls.pdf > 0.0f && !is_black(ls.radiance)) {
            RGB f = bsdf.f<false>(it.wo, ls.wi, flags) * abs_dot(ls.wi, it.ns);
            if (!is_black(f)) {
                float w = power_heuristic(1.0f, ls.pdf, 1.0f, strategy_pdf(ls.wi));
                RGB c = f * ls.radiance * w / ls.pdf;
                Ray sr = spawn_ray_to(it.p, it.p_err, it.n, it.time, ls.pt.p, ls.pt.p_err, ls.pt.n);
                pend[0] = make_float4(c.r, c.g, c.b, 0.0f);
                out.sh_o[0] = make_float4(sr.o.x, sr.o.y, sr.o.z, sr.t_max);
                out.sh_d[0] = make_float4(sr.d.x, sr.d.y, sr.d.z, __int_as_float(-1));
                out.push_sh[0] = true;
                if (chosen && slot < gw.cap) {
                    const float wl = luminance(f * ls.radiance) * count / ls.pdf;
                    if (wl > 0.0f && isfinite(wl)) {
                        float4* r = lrec_ptr(gw, bounce, slot);
                        r[0] = gq.a;
                        r[1] = gq.b;
                        r[2] = make_float4(gq.c.x, ls.wi.x, ls.wi.y, ls.wi.z);
                        r[3] = make_float4(bsdf.pdf<false>(it.wo, ls.wi, flags), 0.0f, wl, 0.0f);
                        state |= ST_LREC;
                    }
                }
            }
        }
        // second strategy: a direction from the BSDF (or the mixture), counted when it reaches the
        // chosen light
        V3 wi;
        RGB f;
        float spdf;
        if (nmix && ug[0] < nmix->c()) {
            wi = nmix->sample(ug[1], ug[2], ug[3]);
            f = bsdf.f<false>(it.wo, wi, flags) * abs_dot(wi, it.ns);
            spdf = strategy_pdf(wi);
        } else {
            BxSample bs = bsdf.sample<false>(it.wo, u[BD_USCAT], u[BD_USCAT + 1], flags);
            wi = bs.wi;
            f = bs.f * abs_dot(bs.wi, it.ns);
            spdf = nmix ? (bs.pdf > 0.0f ? strategy_pdf(bs.wi) : 0.0f) : bs.pdf;
        }
        if (!is_black(f) && spdf > 0.0f) {
            float t_light = 0.0f;
            V3 ln;
            float lpdf = INF ? light_pdf_any<false, SHL>(sc, light_prim, it, wi, &t_light, &ln)
                             : light_pdf<false, false>(sc, light_prim, it, wi, &t_light, &ln);
            if (lpdf != 0.0f) {
                float w = power_heuristic(1.0f, spdf, 1.0f, lpdf);
                // the sampled direction reaches the light at t_light; it counts iff nothing else
                // is hit first (closest hit == this light; for the infinite light t_light is
                // infinite and nothing may be hit)
                RGB li = INF ? light_radiance_along(sc, light_prim, wi, ln)
                             : emission(sc.emis[prim_emission(sc, (int)light_prim)], ln, -wi);
                if (!is_black(li)) {
                    RGB c = f * li * w / spdf;
                    Ray br = spawn_ray(it.p, it.p_err, it.n, it.time, wi, false);
                    pend[1] = make_float4(c.r, c.g, c.b, 0.0f);
                    out.sh_o[1] = make_float4(br.o.x, br.o.y, br.o.z, t_light);
                    const int skip = INF && light_prim == LIGHT_INFINITE ? -1 : (int)light_prim;
                    out.sh_d[1] = make_float4(br.d.x, br.d.y, br.d.z, __int_as_float(skip));
                    out.push_sh[1] = true;
                }
            }
        }
        wb.pending[2 * slot] = pend[0];
        wb.pending[2 * slot + 1] = pend[1];
        wb.nee_beta[slot] = make_float4(beta.r, beta.g, beta.b, 0.0f);
        state |= ST_PENDING;
    }
    V3 wo = -ray.d;
    BxSample bs;
    float p_b;  // BSDF pdf of the continuation (the training record's)
    if (GUIDABLE && mix && (gw.flags & GW_CONT) && bsdf.num_components(BSDF_SPECULAR) == 0) {
        // one-sample MIS: with probability c the direction comes from the guide, else from the
        // BSDF; either way the throughput divides by the mixture pdf c q(wi) + (1 - c) p_bsdf(wi)
        const float c = mix->c();
        const bool from_guide = ug[4] < c;
        if (from_guide) {
            bs.wi = mix->sample(ug[5], ug[6], ug[7]);
            bs.f = bsdf.f<false>(wo, bs.wi, BSDF_ALL);
            p_b = bsdf.pdf<false>(wo, bs.wi, BSDF_ALL);
            bs.stype = BSDF_REFLECTION | BSDF_GLOSSY;  // guidable BSDFs have no specular lobe
        } else {
            bs = bsdf.sample<false>(wo, u[BD_BSDF], u[BD_BSDF + 1], BSDF_ALL);
            p_b = bs.pdf;
        }
        bs.pdf = from_guide || p_b > 0.0f ? c * mix->pdf(bs.wi) + (1.0f - c) * p_b : 0.0f;
    } else {
        bs = bsdf.sample<false>(wo, u[BD_BSDF], u[BD_BSDF + 1], BSDF_ALL);
        p_b = bs.pdf;
    }
    if (is_black(bs.f) || bs.pdf == 0.0f) {
        out.finished = true;
        return;
    }
    RGB beta0 = beta;
    beta = beta * (bs.f * abs_dot(bs.wi, it.ns) / bs.pdf);
    bool spec = (bs.stype & BSDF_SPECULAR) != 0;
    if (spec && (bs.stype & BSDF_TRANSMISSION)) {
        float eta = bsdf.eta;
        eta_scale *= dot(wo, it.n) > 0.0f ? eta * eta : 1.0f / (eta * eta);
    }
    Ray nr = spawn_ray(it.p, it.p_err, it.n, it.time, bs.wi, false);
    RGB rr_beta = beta * eta_scale;
    if (max_value(rr_beta) < rp.rr_threshold && bounce > 3) {
        state = st_set_k(state, st_k1(state) + 1u, st_k2(state));
        float qq = rmax(1.0f - max_value(rr_beta), 0.5f);
        if (u[BD_RR] < qq) {
            out.finished = true;
            return;
        }
        beta = beta / (1.0f - qq);
    }
    wb.ray_o[slot] = make_float4(nr.o.x, nr.o.y, nr.o.z, nr.t_max);
    wb.ray_d[slot] = make_float4(nr.d.x, nr.d.y, nr.d.z, nr.time);
    state = (state & ~(0xFFu | ST_SPECULAR)) | ((bounce + 1) & 0xFFu) | (spec ? ST_SPECULAR : 0u);
    // every positive-weight record of a chosen path enters the pool
    if (chosen) state = open_record(gw, wb, slot, state, gq, bs.wi, p_b, beta0);
    out.cont = true;
}

// Warp-convergent tail of k_shade: queue compaction, shadow rays, records.
// lrec: this lane's path resolved a visible light-sample record of its previous vertex.
BG_D void finish_vertex(const WaveBuffers& wb, const GuideWave& gw, uint32_t bounce, uint32_t slot, bool cont,
                        bool done_pending, const VertexOut& vo, uint32_t emit_n, RGB L_emit, bool record,
                        uint32_t* err, bool lrec = false) {
    uint32_t pos = warp_append(&wb.counters[(bounce + 1) & 1], cont);
    if (cont) wb.queue[(bounce + 1) & 1][pos] = slot;
    pos = warp_append(&wb.counters[C_DONE], done_pending);
    if (done_pending) wb.done[pos] = slot;
    for (int k = 0; k < 2; ++k) {
        pos = warp_append(&wb.counters[C_SHADOW], vo.push_sh[k]);
        if (vo.push_sh[k]) {
            if (pos < wb.sh_capacity) {
                wb.sh_o[pos] = vo.sh_o[k];
                wb.sh_d[pos] = vo.sh_d[k];
                wb.sh_ref[pos] = 2 * slot + (uint32_t)k;
            } else {
                atomicOr(err, ERR_QUEUE_OVERFLOW);
            }
        }
    }
    if (record) {
        emit_records(gw, wb, slot, emit_n, L_emit);
        if (bounce > 0) emit_light_record(gw, bounce - 1, slot, lrec);
    }
}

// Shades the paths of one material class (CLS = bg_material_type, or CLS_MISS for escaped rays).
// In guided waves the matte / plastic / conductor classes read the network's mixture for their
// queue position (inferred after binning, before this launch) and sample with it.
// GWK: guiding support compiled in (records, mixtures); the plain wavefront uses GWK = false.
// Minimum resident CTAs per SM the shade kernels are compiled for: 4 caps them at 128 registers
// (the plastic and conductor classes would use 148 / 159).  Measured on the production scene at
// 4 spp: shade 7.1 ms against 7.7 ms unconstrained; 5 and 6 CTAs gave 7.3 and 7.1 ms.
#ifndef BG_SHADE_MINBLOCKS
#define BG_SHADE_MINBLOCKS 4
#endif
// The guided variants hold the mixture views and eight more uniforms; they are compiled for
// BG_GUIDED_SHADE_MINBLOCKS CTAs per SM (4: matte, plastic and conductor spill 36, 32, 44 bytes).
#ifndef BG_GUIDED_SHADE_MINBLOCKS
#define BG_GUIDED_SHADE_MINBLOCKS 4
#endif
template <int CLS, bool MULTI = false, bool GWK = false, bool TEX = false, bool INF = false, bool SHL = INF>
__global__ void __launch_bounds__(128, GWK ? BG_GUIDED_SHADE_MINBLOCKS : BG_SHADE_MINBLOCKS) k_shade(Scene sc0, RenderParams rp0, FilmBuffers film0, WaveBuffers wb,
                                               GuideWave gw, uint32_t bounce, uint32_t* err, const SceneRender* tab) {
    constexpr bool GUIDABLE = CLS >= 0 && CLS <= 2;
    const uint32_t n = wb.counters[C_CLS + CLS];
    const uint32_t* q = wb.cls_queue + (size_t)CLS * wb.capacity;
    const uint32_t stride = gridDim.x * blockDim.x;
    __shared__ float strat_su[CLS != CLS_MISS ? 8 * SU_STRIDE : 1];
    const bool record = GWK && (gw.flags & GW_RECORD) != 0;
    const bool guided = GWK && GUIDABLE && (gw.flags & GW_GUIDED);
    // warp-uniform loop so the ballots below see all 32 lanes
    for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < n; base += stride) {
        uint32_t i = base + lane_id();
        bool active = i < n;
        uint32_t slot = active ? q[i] : 0;
        bool cont = false, done_pending = false, lrec_emit = false;
        VertexOut vo;
        uint32_t emit_n = 0;
        RGB L_emit = rgb(0.0f);
        if (active) {
            const SceneRender* sr = MULTI ? tab + wb.scene_id[slot] : nullptr;
            const Scene& sc = pick<MULTI>(sc0, MULTI ? &sr->sc : nullptr);
            const RenderParams& rp = pick<MULTI>(rp0, MULTI ? &sr->rp : nullptr);
            const FilmBuffers& film = pick<MULTI>(film0, MULTI ? &sr->film : nullptr);
            float4 ro = wb.ray_o[slot], rd = wb.ray_d[slot];
            Ray ray = load_ray(ro, rd);
            int prim = wb.hit[slot].x;
            uint32_t state = wb.state[slot];
            float4 b4 = wb.beta[slot];
            RGB beta = rgb(b4.x, b4.y, b4.z);
            float eta_scale = b4.w;
            const float* su = nullptr;
            if (CLS != CLS_MISS && rp.strat.dims > 0) {
                float* col = strat_su + threadIdx.x;
                strat_prefetch(rp.strat, wb.pixel[slot], wb.sample[slot], rp.seed, st_k1(state), st_k2(state), col);
                su = col;
            }
            float4 l4 = wb.L[slot];
            RGB L = apply_pending(wb, slot, rgb(l4.x, l4.y, l4.z), state, sc.nlights);
            // the previous vertex's light-sample record: its shadow ray has been traced
            if (record && (state & ST_LREC)) lrec_emit = wb.pending[2 * slot].w != 0.0f;
            state &= ~(ST_PENDING | ST_LREC);
            bool specular_bounce = (state & ST_SPECULAR) != 0;
            Isect it;
            bool hit = CLS != CLS_MISS && prim >= 0 && prim_isect(sc, prim, ray, &it);
            const bool counted = bounce == 0 || specular_bounce;
            const bool rec_open = record && (state & ST_REC_OPEN);
            RGB le = hit && (counted || rec_open) ? emitted_radiance(sc, it, -ray.d) : rgb(0.0f);
            // an escaped ray gathers the infinite light's radiance (path.rs:78-85)
            if (CLS == CLS_MISS && prim < 0 && (counted || rec_open) && sc.inf) le = inf_radiance(sc, ray.d);
            // The previous vertex's record closes here, with this emission as its direct target
            // (which the estimator leaves to that vertex's next-event estimation unless counted).
            if (record) state = close_record(gw, wb, slot, state, counted ? L + beta * le : L, beta * le);
            if (counted) L = L + beta * le;
            bool finished = !hit || bounce >= rp.max_depth;
            if (!finished) {
                // guided: the mixture inferred for this queue position (GW_CONT / GW_NEE place it)
                const bool gv = guided && i < gw.cap;
                const MixView mix{gv ? gw.raw + ((size_t)(GUIDABLE ? CLS : 0) * gw.cap + i) * GUIDE_MIX_HEAD : nullptr};
                float ug[8];
                if (gv) {
                    const Rng grng{wb.pixel[slot], wb.sample[slot], rp.seed};
                    grng.block(DIM_GUIDE0 + 8 * bounce, ug);
                    grng.block(DIM_GUIDE0 + 8 * bounce + 4, ug + 4);
                }
                scatter_vertex<CLS, TEX, INF, SHL>(sc, rp, wb, gw, slot, bounce, ray, it, beta, eta_scale, state,
                                                   gv ? &mix : nullptr, ug, record, vo, su);
                finished = vo.finished;
                cont = vo.cont;
            }
            wb.state[slot] = state;
            wb.beta[slot] = make_float4(beta.r, beta.g, beta.b, eta_scale);
            wb.L[slot] = make_float4(L.r, L.g, L.b, 0.0f);
            if (finished) {
                if (state & ST_PENDING) {
                    done_pending = true;
                } else {
                    film_add(film, wb.pixel[slot], L);
                    emit_n = rec_count(state);
                    L_emit = L;
                }
            }
        }
        finish_vertex(wb, gw, bounce, slot, cont, done_pending, vo, emit_n, L_emit, record, err, lrec_emit);
    }
}

// Streams of one bounce's class kernels.  The classes share no data a kernel of another class
// reads (each shades its own queue's paths, writes only those paths' slots and appends to the next
// queues and the training pool with atomics), so with a fork they run side by side: matte (the
// largest class) on the launching stream, plastic, conductor, dielectric and the misses on the
// fork's streams, which first wait for everything already on `s`; shade_join makes `s` wait for
// them again.
struct ClassStreams {
    cudaStream_t st[5];  // by class: matte, plastic, conductor, dielectric, misses
};
inline ClassStreams shade_fork(cudaStream_t s, const ShadeFork* fork) {
    ClassStreams cs{{s, s, s, s, s}};
    if (fork) {
        cudaEventRecord(fork->fork, s);
        for (int k = 0; k < 4; ++k) {
            cudaStreamWaitEvent(fork->aux[k], fork->fork, 0);
            cs.st[1 + k] = fork->aux[k];
        }
    }
    return cs;
}
inline void shade_join(cudaStream_t s, const ShadeFork* fork) {
    if (!fork) return;
    for (int k = 0; k < 4; ++k) {
        cudaEventRecord(fork->join[k], fork->aux[k]);
        cudaStreamWaitEvent(s, fork->join[k], 0);
    }
}

// Single-scene shade launches for scenes with emitting spheres or quadrics (bg_shade_shapes.cu).
int launch_shade_shapes(const Scene& sc, const RenderParams& rp, const FilmBuffers& film, const WaveBuffers& wb,
                        uint32_t bounce, uint32_t* err, dim3 grid, dim3 block, cudaStream_t s);
// Shade launches of one bounce (the five material classes, misses included); with `fork` the
// classes run on parallel streams, joined back into `s` before returning.
int launch_shade_plain(const Scene& sc, const RenderParams& rp, const FilmBuffers& film, const WaveBuffers& wb,
                       uint32_t bounce, uint32_t* err, dim3 grid, dim3 block, cudaStream_t s,
                       const ShadeFork* fork = nullptr);
int launch_shade_guided(const Scene& sc, const RenderParams& rp, const FilmBuffers& film, const WaveBuffers& wb,
                        const GuideWave& gw, uint32_t bounce, uint32_t* err, dim3 grid, dim3 block, cudaStream_t s,
                        const ShadeFork* fork = nullptr);
// The guided launches of scenes with textures or an infinite light (bg_shade_guided_full.cu).
int launch_shade_guided_full(const Scene& sc, const RenderParams& rp, const FilmBuffers& film, const WaveBuffers& wb,
                             const GuideWave& gw, uint32_t bounce, uint32_t* err, dim3 grid, dim3 block,
                             cudaStream_t s, const ShadeFork* fork = nullptr);
// full: the variants that handle textured scenes and infinite lights (checked per path's scene).
int launch_shade_batch(const SceneRender* tab, const WaveBuffers& wb, uint32_t bounce, uint32_t* err, dim3 grid,
                       dim3 block, cudaStream_t s, bool full);

}  // namespace bg

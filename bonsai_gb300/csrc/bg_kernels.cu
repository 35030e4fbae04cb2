// bg_kernels.cu - ray-query kernels, the per-path megakernel and the PBRT wavefront stages.
//
// Wavefront (PBRT mode, 2-wide BVH):  one wave = up to `capacity` (pixel, sample) paths.
//   generate -> [prepare -> extend -> shade -> shadow -> finalize] x (max_depth + 1)
// Queue sizes live in device memory; every stage launches a fixed persistent grid that reads its
// own work count, so the chain needs no host synchronisation and can be captured in a CUDA graph.
// Traversal stages pull 32-ray batches per warp from an atomic head (dynamic load balance);
// queues are compacted with warp ballot + popc + one atomic per warp.
//
// Megakernel (both modes, reference-layout BVH): one thread per (pixel, sample) runs
// PathIntegrator::radiance end to end; it is the REF_COMPAT path and a cross-check of the
// wavefront in PBRT mode.
#include "bg_guide.cuh"
#include "bg_guide_kernels.h"
#include "bg_kernels.h"
#include "bg_shading.cuh"
#include "bg_traverse.cuh"
#include "bg_film.cuh"
#include "bg_estimate.cuh"
#include "bg_warp.cuh"
#include "bg_wave.cuh"

namespace bg {


// ================================================================ ray queries
struct TraceSrc {
    const float4* rays;
    int2* hits;
    uint8_t* occ;
    BG_D Ray load(uint32_t i, int* skip) const {
        Ray r = load_ray(__ldg(&rays[2 * i]), __ldg(&rays[2 * i + 1]));
        r.time = 0.0f;
        *skip = -1;
        return r;
    }
    BG_D void store(uint32_t i, int prim, float t) const {
        if (occ) occ[i] = prim >= 0 ? 1 : 0;
        else hits[i] = make_int2(prim, __float_as_int(prim >= 0 ? t : INFINITY));
    }
};

// LAYOUT: 1 = reference binary layout, 2 = 2-wide, 8 = 8-wide compressed.
// Traversal kernels are capped at 64 registers (8 blocks of 128 threads per SM): occupancy hides
// the node-fetch latency better than the extra registers would (measured on the production scene:
// -20% frame time against the uncapped 96-register build).
#ifndef BG_MINBLOCKS
#define BG_MINBLOCKS 8
#endif
template <int LAYOUT, bool ANY>
__global__ void __launch_bounds__(128, BG_MINBLOCKS) k_trace(Scene sc, const float4* rays, uint32_t n, int2* hits, uint8_t* occ,
                                               uint32_t* err, unsigned long long* counters, uint32_t* head, int refill) {
    if constexpr (LAYOUT != 1) {
        TraceSrc src{rays, hits, ANY ? occ : nullptr};
#if BG_SMEM_STACK
        __shared__ uint2 stack8[STACK8 * 128];
#else
        uint2* stack8 = nullptr;
#endif
        if (LAYOUT == 8) traverse_queue8<ANY>(sc, n, head, src, err, refill, stack8);
        else traverse_queue<ANY>(sc, n, head, src, err, refill);
        return;
    } else {
        for (;;) {
            uint32_t base = warp_fetch(head);
            if (base >= n) break;
            uint32_t i = base + lane_id();
            if (i < n) {
                Ray ray = load_ray(__ldg(&rays[2 * i]), __ldg(&rays[2 * i + 1]));
                ray.time = 0.0f;
                int prim = ref_traverse<ANY>(sc, ray, err, counters);
                if (ANY) occ[i] = prim >= 0 ? 1 : 0;
                else hits[i] = make_int2(prim, __float_as_int(prim >= 0 ? ray.t_max : INFINITY));
            }
        }
    }
}

void launch_trace(const Scene& sc, bool ref_layout, bool any, const bg_ray* rays, size_t n, bg_hit* hits,
                  uint8_t* occluded, uint32_t* err, unsigned long long* counters, uint32_t* work_head,
                  const LaunchShape& ls, cudaStream_t s) {
    cudaMemsetAsync(work_head, 0, sizeof(uint32_t), s);
    dim3 grid(ls.sms * ls.blocks_per_sm), block(128);
    const float4* r = reinterpret_cast<const float4*>(rays);
    int2* h = reinterpret_cast<int2*>(hits);
    uint32_t nn = (uint32_t)n;
    const int layout = ref_layout ? 1 : (sc.nodes8 ? 8 : 2);
#define BG_TRACE(L, A) k_trace<L, A><<<grid, block, 0, s>>>(sc, r, nn, h, occluded, err, counters, work_head, ls.refill)
    if (layout == 1) {
        if (any) BG_TRACE(1, true);
        else BG_TRACE(1, false);
    } else if (layout == 2) {
        if (any) BG_TRACE(2, true);
        else BG_TRACE(2, false);
    } else {
        if (any) BG_TRACE(8, true);
        else BG_TRACE(8, false);
    }
#undef BG_TRACE
}

// ================================================================ megakernel (reference layout)
// `rd0`: the camera ray's differentials (textured scenes), which the path keeps in REF mode (the
// ray never re-spawns, F1) and only has at the first hit in PBRT mode.
template <bool REF>
BG_D RGB radiance_ref(const Scene& sc, Ray ray, const Rng& rng, uint32_t max_depth, float rr_threshold,
                      uint32_t* err, const RayDiff* rd0, const StratParams& sp) {
    SamplerCalls calls{sp, REF, rng.pixel, rng.sample, rng.seed, 1u, 2u};  // after the camera sample
    RGB out = rgb(0.0f), beta = rgb(1.0f);
    bool specular_bounce = false;
    float eta_scale = 1.0f;
    for (uint32_t bounces = 0;; ++bounces) {
        Ray traced = ray;
        int prim = ref_traverse<false>(sc, ray, err, nullptr);  // sets ray.t_max to the hit
        bool hit = prim >= 0;
        Isect it;
        if (hit) hit = prim_isect(sc, prim, traced, &it);
        if (bounces == 0 || specular_bounce) {
            if (hit) out = out + beta * emitted_radiance(sc, it, -ray.d);
            else if (prim < 0) out = out + beta * escaped_radiance(sc, ray.d);
        }
        if (!hit || bounces >= max_depth) break;
        TexPoint tp;
        BSDF bsdf = make_bsdf<-1, REF>(sc, it, tex_point(sc, it, traced, (REF || bounces == 0) ? rd0 : nullptr, &tp));
        const uint32_t base = DIM_BOUNCE0 + DIMS_PER_BOUNCE * bounces;
        float u[8];
        rng.block(base, u);
        rng.block(base + 4, u + 4);
        if (bsdf.num_components(BSDF_ALL & ~BSDF_SPECULAR) > 0 && sc.nlights > 0) {
            calls.get_1d(u[BD_LIGHT]);
            calls.get_2d(u[BD_ULIGHT], u[BD_ULIGHT + 1]);
            calls.get_2d(u[BD_USCAT], u[BD_USCAT + 1]);
            float count = (float)sc.nlights;
            uint32_t li = (uint32_t)rmin(u[BD_LIGHT] * count, count - 1.0f);
            float lpdf = 1.0f / count;
            RGB ld = estimate_direct_mk<REF, 1>(sc, it, bsdf, sc.light_prims[li], u[BD_USCAT], u[BD_USCAT + 1],
                                              u[BD_ULIGHT], u[BD_ULIGHT + 1], err);
            out = out + beta * (ld / lpdf);
        }
        V3 wo = -ray.d;
        calls.get_2d(u[BD_BSDF], u[BD_BSDF + 1]);
        BxSample bs = bsdf.sample<REF>(wo, u[BD_BSDF], u[BD_BSDF + 1], BSDF_ALL);
        if (is_black(bs.f) || bs.pdf == 0.0f) break;
        beta = beta * (bs.f * abs_dot(bs.wi, it.ns) / bs.pdf);
        specular_bounce = (bs.stype & BSDF_SPECULAR) != 0;
        if ((bs.stype & BSDF_SPECULAR) && (bs.stype & BSDF_TRANSMISSION)) {
            float eta = bsdf.eta;
            eta_scale *= dot(wo, it.n) > 0.0f ? eta * eta : 1.0f / (eta * eta);
        }
        // F1: REF re-intersects the same ray (t_max already at this hit); PBRT moves on
        if (!REF) ray = spawn_ray(it.p, it.p_err, it.n, it.time, bs.wi, false);
        RGB rr_beta = beta * eta_scale;
        if (max_value(rr_beta) < rr_threshold && bounces > 3) {
            calls.get_1d(u[BD_RR]);
            float q = rmax(1.0f - max_value(rr_beta), 0.5f);
            if (u[BD_RR] < q) break;
            beta = beta / (1.0f - q);
        }
    }
    return out;
}

template <bool REF>
__global__ void __launch_bounds__(128) k_megakernel(Scene sc, Camera cam, RenderParams rp, FilmBuffers film,
                                                    uint32_t* err) {
    const uint64_t npix = (uint64_t)rp.width * rp.height;
    const uint64_t total = npix * rp.spp;
    for (uint64_t item = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; item < total;
         item += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t pix = (uint32_t)(item % npix);
        uint32_t s = rp.first_sample + (uint32_t)(item / npix);
        Rng rng{pix, s, rp.seed};
        const CameraUs cu = camera_us(rp.strat, REF, rng, cam.lens_radius > 0.0f);
        float fx = (float)(pix % rp.width) + cu.fx, fy = (float)(pix / rp.width) + cu.fy;
        Ray ray = camera_ray(cam, fx, fy, cu.time, cu.lx, cu.ly);
        RayDiff rd;
        if (sc.ntex) rd = camera_diff(cam, fx, fy, ray, rp.diff_scale, cu.lx, cu.ly);
        RGB L = radiance_ref<REF>(sc, ray, rng, rp.max_depth, rp.rr_threshold, err, sc.ntex ? &rd : nullptr,
                                  rp.strat);
        film_add(film, pix, L);
    }
}

void launch_megakernel(bool ref_compat, const Scene& sc, const Camera& cam, const RenderParams& rp,
                       const FilmBuffers& film, uint32_t* err, const LaunchShape& ls, cudaStream_t s) {
    dim3 grid(ls.sms * 8), block(128);
    if (ref_compat) k_megakernel<true><<<grid, block, 0, s>>>(sc, cam, rp, film, err);
    else k_megakernel<false><<<grid, block, 0, s>>>(sc, cam, rp, film, err);
}

// Batch: item -> scene by binary search over the scenes' first items, then as above.
__global__ void k_generate_batch(const SceneRender* tab, uint32_t nscenes, WaveBuffers wb, uint64_t item0,
                                 uint32_t nitems) {
    if (blockIdx.x == 0 && threadIdx.x == 0) wb.counters[C_Q0] = nitems;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nitems; i += gridDim.x * blockDim.x) {
        const uint64_t item = item0 + i;
        uint32_t lo = 0, hi = nscenes - 1;
        while (lo < hi) {  // last scene with item0 <= item
            uint32_t mid = (lo + hi + 1) >> 1;
            if (tab[mid].item0 <= item) lo = mid;
            else hi = mid - 1;
        }
        const SceneRender& sr = tab[lo];
        const uint64_t local = item - sr.item0;
        const uint64_t npix = (uint64_t)sr.rp.width * sr.rp.height;
        generate_one(sr.cam, sr.rp, wb, i, (uint32_t)(local % npix), sr.rp.first_sample + (uint32_t)(local / npix));
        wb.scene_id[i] = lo;
    }
}


__global__ void k_generate(Camera cam, RenderParams rp, WaveBuffers wb, uint64_t item0, uint32_t nitems) {
    generate_paths(cam, rp, wb, item0, nitems, rp.first_sample);
}

// Graph replay: the wave to generate comes from wb.wavectl (advanced by k_wave_advance).
__global__ void k_generate_ctl(Camera cam, RenderParams rp, WaveBuffers wb, uint64_t total) {
    const uint64_t item0 = (uint64_t)wb.wavectl[0] * wb.capacity;
    const uint32_t nitems = item0 >= total ? 0u : (uint32_t)min((uint64_t)wb.capacity, total - item0);
    generate_paths(cam, rp, wb, item0, nitems, wb.wavectl[1]);
}

__global__ void k_wave_advance(WaveBuffers wb) {
    if (threadIdx.x == 0) wb.wavectl[0] += 1;
}

__global__ void k_prepare(WaveBuffers wb, uint32_t bounce) {
    if (threadIdx.x == 0) {
        wb.counters[(bounce + 1) & 1] = 0;
        wb.counters[C_SHADOW] = 0;
        wb.counters[C_DONE] = 0;
        wb.counters[C_EXT_HEAD] = 0;
        wb.counters[C_SH_HEAD] = 0;
        for (int c = 0; c < NCLS; ++c) wb.counters[C_CLS + c] = 0;
    }
}

struct ExtendSrc {
    const uint32_t* q;
    WaveBuffers wb;
    const SceneRender* tab;
    BG_D Ray load(uint32_t i, int* skip) const {
        uint32_t slot = q[i];
        *skip = -1;
        return load_ray(wb.ray_o[slot], wb.ray_d[slot]);
    }
    BG_D const Scene* scene(uint32_t i) const { return &tab[wb.scene_id[q[i]]].sc; }
    BG_D void store(uint32_t i, int prim, float t) const { wb.hit[q[i]] = make_int2(prim, __float_as_int(t)); }
};

template <int LAYOUT, bool MULTI = false>
__global__ void __launch_bounds__(128, BG_MINBLOCKS) k_extend(Scene sc, WaveBuffers wb, uint32_t bounce, uint32_t* err,
                                                int refill, const SceneRender* tab, bool sorted) {
    const uint32_t n = wb.counters[bounce & 1];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&wb.ray_stats[0], (unsigned long long)n);
    ExtendSrc src{sorted ? wb.qsort : wb.queue[bounce & 1], wb, tab};
#if BG_SMEM_STACK
    __shared__ uint2 stack8[LAYOUT == 8 ? STACK8 * 128 : 1];
#else
    uint2* stack8 = nullptr;
#endif
    if (LAYOUT == 8) traverse_queue8<false, ExtendSrc, MULTI>(sc, n, &wb.counters[C_EXT_HEAD], src, err, refill, stack8);
    else traverse_queue<false>(sc, n, &wb.counters[C_EXT_HEAD], src, err, refill);
}

// ---- ray binning (BG_TUNE_SORT_RAYS): the extension queue of a bounce, counting-sorted by
// key = direction octant (3 bits) x Morton index of the origin's cell in an 8x8x8 grid over the
// scene bounds (9 bits).  Rays that leave the same region in the same octant then sit in the same
// warps and walk the same part of the tree.  hist: block-local shared-memory counts added to a
// global histogram; scan: one block turns it into bin cursors (and clears the histogram);
// scatter: each block reserves one range per (block, bin) and places its rays by local rank.
constexpr int SORT_BINS = 4096;
constexpr int SORT_K = 8;  // rays per thread per scatter chunk

BG_D uint32_t spread3(uint32_t v) {  // 3 bits -> every third bit
    return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4);
}
BG_D uint32_t ray_key(const WaveBuffers& wb, const RenderParams& rp, uint32_t slot) {
    const float4 o = wb.ray_o[slot], d = wb.ray_d[slot];
    const uint32_t oct = (d.x < 0.0f ? 4u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 1u : 0u);
    const uint32_t cx = (uint32_t)rclamp((o.x - rp.bmin[0]) * rp.binv[0] * 8.0f, 0.0f, 7.0f);
    const uint32_t cy = (uint32_t)rclamp((o.y - rp.bmin[1]) * rp.binv[1] * 8.0f, 0.0f, 7.0f);
    const uint32_t cz = (uint32_t)rclamp((o.z - rp.bmin[2]) * rp.binv[2] * 8.0f, 0.0f, 7.0f);
    return (oct << 9) | (spread3(cx) << 2) | (spread3(cy) << 1) | spread3(cz);
}

__global__ void __launch_bounds__(256) k_sort_hist(WaveBuffers wb, RenderParams rp, uint32_t bounce) {
    __shared__ uint32_t h[SORT_BINS];
    for (int b = threadIdx.x; b < SORT_BINS; b += blockDim.x) h[b] = 0;
    __syncthreads();
    const uint32_t n = wb.counters[bounce & 1];
    const uint32_t* q = wb.queue[bounce & 1];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&h[ray_key(wb, rp, q[i])], 1u);
    __syncthreads();
    for (int b = threadIdx.x; b < SORT_BINS; b += blockDim.x)
        if (h[b]) atomicAdd(&wb.sort_hist[b], h[b]);
}

__global__ void __launch_bounds__(1024) k_sort_scan(WaveBuffers wb) {
    __shared__ uint32_t part[1024];
    constexpr int PER = SORT_BINS / 1024;
    uint32_t v[PER], sum = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        v[k] = wb.sort_hist[threadIdx.x * PER + k];
        sum += v[k];
    }
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {  // inclusive Hillis-Steele scan of the partial sums
        uint32_t x = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += x;
        __syncthreads();
    }
    uint32_t base = part[threadIdx.x] - sum;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        wb.sort_hist[SORT_BINS + threadIdx.x * PER + k] = base;
        wb.sort_hist[threadIdx.x * PER + k] = 0;  // ready for the next bounce
        base += v[k];
    }
}

__global__ void __launch_bounds__(256) k_sort_scatter(WaveBuffers wb, RenderParams rp, uint32_t bounce) {
    __shared__ uint32_t h[SORT_BINS];
    const uint32_t n = wb.counters[bounce & 1];
    const uint32_t* q = wb.queue[bounce & 1];
    uint32_t* cursor = wb.sort_hist + SORT_BINS;
    const uint32_t chunk = blockDim.x * SORT_K;
    for (uint32_t c0 = blockIdx.x * chunk; c0 < n; c0 += gridDim.x * chunk) {
        for (int b = threadIdx.x; b < SORT_BINS; b += blockDim.x) h[b] = 0;
        __syncthreads();
        uint32_t key[SORT_K], rank[SORT_K], slot[SORT_K];
#pragma unroll
        for (int k = 0; k < SORT_K; ++k) {
            const uint32_t i = c0 + k * blockDim.x + threadIdx.x;
            key[k] = SORT_BINS;
            if (i < n) {
                slot[k] = q[i];
                key[k] = ray_key(wb, rp, slot[k]);
                rank[k] = atomicAdd(&h[key[k]], 1u);
            }
        }
        __syncthreads();
        for (int b = threadIdx.x; b < SORT_BINS; b += blockDim.x)
            if (h[b]) h[b] = atomicAdd(&cursor[b], h[b]);  // this block's range of bin b
        __syncthreads();
#pragma unroll
        for (int k = 0; k < SORT_K; ++k)
            if (key[k] < SORT_BINS) {
                const uint32_t pos = h[key[k]] + rank[k];
                if (pos < n) wb.qsort[pos] = slot[k];
            }
        __syncthreads();
    }
}

// Material-key binning of this bounce's hits: one queue per material class plus misses, so each
// shade launch runs one material's code with uniform control flow.  GWK (guided waves, queries
// set): a hit of a guidable class (matte, plastic, conductor) also writes its network query at
// class * gw.cap + its queue position, for the inference that runs before shading.
template <bool MULTI = false, bool GWK = false>
__global__ void __launch_bounds__(128) k_bin(Scene sc0, WaveBuffers wb, uint32_t bounce, const SceneRender* tab,
                                             GuideWave gw = GuideWave{}, bool queries = false) {
    const uint32_t n = wb.counters[bounce & 1];
    const uint32_t* q = wb.queue[bounce & 1];
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < n; base += stride) {
        uint32_t i = base + lane_id();
        int cls = -1;
        uint32_t slot = 0;
        if (i < n) {
            slot = q[i];
            int prim = wb.hit[slot].x;
            const Scene& sc = pick<MULTI>(sc0, MULTI ? &tab[wb.scene_id[slot]].sc : nullptr);
            cls = prim < 0 ? CLS_MISS : (int)sc.prim_cls[prim];
        }
        uint32_t qpos = 0;
#pragma unroll
        for (int c = 0; c < NCLS; ++c) {
            uint32_t pos = warp_append(&wb.counters[C_CLS + c], cls == c);
            if (cls == c) {
                wb.cls_queue[(size_t)c * wb.capacity + pos] = slot;
                qpos = (uint32_t)c * gw.cap + pos;
            }
        }
        // one intersection per lane (outside the class loop, so the lanes of all three classes
        // run it together)
        if (GWK && queries && cls >= 0 && cls <= 2 && qpos - (uint32_t)cls * gw.cap < gw.cap) {
            const Ray ray = load_ray(wb.ray_o[slot], wb.ray_d[slot]);
            Isect it;
            GuideQuery gq{make_float4(0.5f, 0.5f, 0.5f, 0.0f), make_float4(0.0f, 1.0f, 0.0f, 0.0f),
                          make_float4(1.0f, 0.0f, 0.0f, 0.0f)};
            if (prim_isect(sc0, wb.hit[slot].x, ray, &it)) gq = make_query(gw, it, -ray.d);
            float4* o = gw.query + 3 * (size_t)qpos;
            o[0] = gq.a;
            o[1] = gq.b;
            o[2] = gq.c;
        }
    }
}

struct ShadowSrc {
    WaveBuffers wb;
    const SceneRender* tab;
    BG_D const Scene* scene(uint32_t i) const { return &tab[wb.scene_id[wb.sh_ref[i] >> 1]].sc; }
    BG_D Ray load(uint32_t i, int* skip) const {
        float4 o = wb.sh_o[i], d = wb.sh_d[i];
        Ray ray;
        ray.o = f4xyz(o);
        ray.t_max = o.w;
        ray.d = f4xyz(d);
        ray.time = 0.0f;
        *skip = __float_as_int(d.w);
        return ray;
    }
    BG_D void store(uint32_t i, int prim, float) const {
        if (prim < 0) wb.pending[wb.sh_ref[i]].w = 1.0f;
    }
};

template <int LAYOUT, bool MULTI = false>
__global__ void __launch_bounds__(128, BG_MINBLOCKS) k_shadow(Scene sc, WaveBuffers wb, uint32_t* err, int refill,
                                                              const SceneRender* tab) {
    const uint32_t n = min(wb.counters[C_SHADOW], wb.sh_capacity);
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&wb.ray_stats[1], (unsigned long long)n);
    ShadowSrc src{wb, tab};
#if BG_SMEM_STACK
    __shared__ uint2 stack8[LAYOUT == 8 ? STACK8 * 128 : 1];
#else
    uint2* stack8 = nullptr;
#endif
    if (LAYOUT == 8) traverse_queue8<true, ShadowSrc, MULTI>(sc, n, &wb.counters[C_SH_HEAD], src, err, refill, stack8);
    else traverse_queue<true>(sc, n, &wb.counters[C_SH_HEAD], src, err, refill);
}

template <bool MULTI = false, bool GWK = false>
__global__ void __launch_bounds__(128) k_finalize(Scene sc0, FilmBuffers film0, WaveBuffers wb, GuideWave gw,
                                                  const SceneRender* tab, uint32_t bounce = 0) {
    const uint32_t n = wb.counters[C_DONE];
    const bool record = GWK && (gw.flags & GW_RECORD) != 0;
    for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < n; base += gridDim.x * blockDim.x) {
        uint32_t i = base + lane_id();
        uint32_t slot = 0, nrec = 0;
        bool lrec = false;
        RGB L = rgb(0.0f);
        if (i < n) {
            slot = wb.done[i];
            const SceneRender* sr = MULTI ? tab + wb.scene_id[slot] : nullptr;
            const Scene& sc = pick<MULTI>(sc0, MULTI ? &sr->sc : nullptr);
            const FilmBuffers& film = pick<MULTI>(film0, MULTI ? &sr->film : nullptr);
            float4 l4 = wb.L[slot];
            uint32_t state = wb.state[slot];
            L = apply_pending(wb, slot, rgb(l4.x, l4.y, l4.z), state, sc.nlights);
            film_add(film, wb.pixel[slot], L);
            nrec = rec_count(state);
            // the last vertex's light-sample record, resolved by this bounce's shadow rays
            lrec = record && (state & ST_LREC) && wb.pending[2 * slot].w != 0.0f;
        }
        if (record) {
            emit_records(gw, wb, slot, nrec, L);
            emit_light_record(gw, bounce, slot, lrec);
        }
    }
}

static int launch_bounces(const Scene& sc, const RenderParams& rp, const FilmBuffers& film, const WaveBuffers& wb,
                          uint32_t* err, const LaunchShape& ls, cudaStream_t s, cudaEvent_t* ev, const GuideWave* gwp) {
    int launches = 0;
    dim3 grid(ls.sms * ls.blocks_per_sm), block(128);
    const GuideWave gw = gwp ? *gwp : GuideWave{};
    const bool guided = (gw.flags & GW_GUIDED) != 0;
    for (uint32_t b = 0; b <= rp.max_depth; ++b) {
        k_prepare<<<1, 32, 0, s>>>(wb, b);
        if (ev) cudaEventRecord(ev[4 * b + 0], s);
        const bool sorted = ls.sort_rays && b > 0 && wb.qsort;
        if (sorted) {
            k_sort_hist<<<ls.sms * 4, 256, 0, s>>>(wb, rp, b);
            k_sort_scan<<<1, 1024, 0, s>>>(wb);
            k_sort_scatter<<<ls.sms * 4, 256, 0, s>>>(wb, rp, b);
            launches += 3;
        }
        if (sc.nodes8) k_extend<8><<<grid, block, 0, s>>>(sc, wb, b, err, ls.refill, nullptr, sorted);
        else k_extend<2><<<grid, block, 0, s>>>(sc, wb, b, err, ls.refill, nullptr, sorted);
        const bool queries = guided && b < rp.max_depth;
        if (queries) {
            // every hit of a guidable class queues its network query; the network's mixtures are
            // ready before the shade launches
            k_bin<false, true><<<grid, block, 0, s>>>(sc, wb, b, nullptr, gw, true);
            launch_guide_infer(gw.wpack, gw.query, &wb.counters[C_CLS], 3, gw.cap, gw.raw, true, err, ls.sms, s);
            launches += 1;
        } else {
            k_bin<<<grid, block, 0, s>>>(sc, wb, b, nullptr);
        }
        if (ev) cudaEventRecord(ev[4 * b + 1], s);
        if (gw.flags) launches += launch_shade_guided(sc, rp, film, wb, gw, b, err, grid, block, s, ls.fork);
        else launches += launch_shade_plain(sc, rp, film, wb, b, err, grid, block, s, ls.fork);
        if (ev) cudaEventRecord(ev[4 * b + 2], s);
        if (sc.nodes8) k_shadow<8><<<grid, block, 0, s>>>(sc, wb, err, ls.refill, nullptr);
        else k_shadow<2><<<grid, block, 0, s>>>(sc, wb, err, ls.refill, nullptr);
        if (ev) cudaEventRecord(ev[4 * b + 3], s);
        if (gw.flags) k_finalize<false, true><<<grid, block, 0, s>>>(sc, film, wb, gw, nullptr, b);
        else k_finalize<<<grid, block, 0, s>>>(sc, film, wb, gw, nullptr);
        launches += 5;
    }
    return launches;
}

int launch_wave(const Scene& sc, const Camera& cam, const RenderParams& rp, const FilmBuffers& film,
                const WaveBuffers& wb, uint64_t item0, uint32_t nitems, uint32_t* err, const LaunchShape& ls,
                cudaStream_t s, cudaEvent_t* ev, const GuideWave* gw) {
    dim3 grid(ls.sms * ls.blocks_per_sm), block(128);
    k_generate<<<grid, block, 0, s>>>(cam, rp, wb, item0, nitems);
    return 1 + launch_bounces(sc, rp, film, wb, err, ls, s, ev, gw);
}

int launch_wave_batch(const SceneRender* tab, uint32_t nscenes, uint32_t max_depth, const WaveBuffers& wb,
                      uint64_t item0, uint32_t nitems, uint32_t* err, const LaunchShape& ls, cudaStream_t s,
                      uint32_t variants) {
    dim3 grid(ls.sms * ls.blocks_per_sm), block(128);
    const Scene sc{};
    const FilmBuffers film{};
    const GuideWave gw{};
    k_generate_batch<<<grid, block, 0, s>>>(tab, nscenes, wb, item0, nitems);
    int launches = 1;
    for (uint32_t b = 0; b <= max_depth; ++b) {
        k_prepare<<<1, 32, 0, s>>>(wb, b);
        k_extend<8, true><<<grid, block, 0, s>>>(sc, wb, b, err, ls.refill, tab, false);
        k_bin<true><<<grid, block, 0, s>>>(sc, wb, b, tab);
        launch_shade_batch(tab, wb, b, err, grid, block, s, variants != 0);
        k_shadow<8, true><<<grid, block, 0, s>>>(sc, wb, err, ls.refill, tab);
        k_finalize<true><<<grid, block, 0, s>>>(sc, film, wb, gw, tab);
        launches += 10;
    }
    return launches;
}

int launch_wave_chain(const Scene& sc, const Camera& cam, const RenderParams& rp, const FilmBuffers& film,
                      const WaveBuffers& wb, uint64_t total, uint32_t* err, const LaunchShape& ls, cudaStream_t s) {
    dim3 grid(ls.sms * ls.blocks_per_sm), block(128);
    k_generate_ctl<<<grid, block, 0, s>>>(cam, rp, wb, total);
    int n = 1 + launch_bounces(sc, rp, film, wb, err, ls, s, nullptr, nullptr);
    k_wave_advance<<<1, 32, 0, s>>>(wb);
    return n + 1;
}

// ================================================================ film
__global__ void k_resolve(FilmBuffers f) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < f.npix; p += gridDim.x * blockDim.x) {
        // merge_film_tile's rgb_to_xyz (film.rs:138-154) then write_image (film.rs:156-202)
        float r = (float)f.sum[3 * p], g = (float)f.sum[3 * p + 1], b = (float)f.sum[3 * p + 2];
        float X = 0.412453f * r + 0.357580f * g + 0.180423f * b;
        float Y = 0.212671f * r + 0.715160f * g + 0.072169f * b;
        float Z = 0.019334f * r + 0.119193f * g + 0.950227f * b;
        float o0 = 3.240479f * X - 1.537150f * Y - 0.498535f * Z;
        float o1 = -0.969256f * X + 1.875991f * Y + 0.041556f * Z;
        float o2 = 0.055648f * X - 0.204043f * Y + 1.057311f * Z;
        float w = (float)f.count[p];
        if (w != 0.0f) {
            float inv = 1.0f / w;
            o0 = fmaxf(o0 * inv, 0.0f);
            o1 = fmaxf(o1 * inv, 0.0f);
            o2 = fmaxf(o2 * inv, 0.0f);
        }
        f.rgb[3 * p] = o0;
        f.rgb[3 * p + 1] = o1;
        f.rgb[3 * p + 2] = o2;
    }
}

void launch_resolve(const FilmBuffers& film, cudaStream_t s) {
    k_resolve<<<(film.npix + 255) / 256, 256, 0, s>>>(film);
}

void launch_clear_film(const FilmBuffers& film, cudaStream_t s) {
    cudaMemsetAsync(film.sum, 0, sizeof(double) * 3 * film.npix, s);
    cudaMemsetAsync(film.sumsq, 0, sizeof(double) * 3 * film.npix, s);
    cudaMemsetAsync(film.count, 0, sizeof(uint32_t) * film.npix, s);
}

}  // namespace bg

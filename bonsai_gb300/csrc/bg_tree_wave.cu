// bg_tree_wave.cu - the Whitted and direct-lighting ray trees as a breadth-first wavefront.
//
// A camera sample's radiance in WhittedIntegrator / DirectLightingIntegrator
// (src/integrators/{whitted,direct}.rs, src/base/integrator.rs:143-307) is a tree: every node
// (a ray) adds its hit's emission and light samples, and a specular hit spawns a reflected and a
// transmitted child.  Glass makes the trees uneven (one node for a diffuse pixel, tens behind a
// glass object), so one thread per sample leaves most lanes of a warp idle.  Here every node is a
// work item instead: level d of all the wave's trees is one queue, traced by the persistent
// traversal with warp refill, shaded (emission, light-sampling rays into the shadow queue,
// children into the level-(d+1) queue), and its shadow rays are traced as one any-hit batch.
// Contributions add into per-sample accumulators; the film receives each sample's total, after
// SamplerIntegrator::render's sanity checks, when the wave's trees are done.
//
// Random numbers, dimensions and node ids are those of the per-sample kernel (bg_integrators.cu),
// so both produce the same estimate for every sample up to float summation order.  The direct
// strategy of MIS through the BSDF becomes an occlusion ray up to the light (the light's own
// triangle skipped), as in the path wavefront.
#include "bg_tree_wave.cuh"

#ifndef BG_MINBLOCKS
#define BG_MINBLOCKS 8
#endif

namespace bg {

// The wave's camera samples as the level-0 nodes (node id 1, depth 0).
__global__ void k_tw_gen(Camera cam, RenderParams rp, TreeWave tw, uint64_t item0, uint32_t n) {
    const uint64_t npix = (uint64_t)rp.width * rp.height;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        tw.counters[0] = n;
        tw.counters[1] = 0;
        tw.counters[TW_SHADOW] = 0;
        tw.counters[TW_EXT_HEAD] = 0;
        tw.counters[TW_SH_HEAD] = 0;
        tw.counters[TW_OVERFLOW] = 0;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint64_t item = item0 + i;
        const uint32_t pix = pixel_of((uint32_t)(item % npix), rp.width, rp.height, rp.pixel_tiles);
        const uint32_t s = rp.first_sample + (uint32_t)(item / npix);
        const Rng rng{pix, s, rp.seed, 0u};
        const CameraUs cu = camera_us(rp.strat, false, rng, cam.lens_radius > 0.0f);  // sampled_dimensions <= 1: camera only
        const float fx = (float)(pix % rp.width) + cu.fx, fy = (float)(pix / rp.width) + cu.fy;
        const Ray r = camera_ray(cam, fx, fy, cu.time, cu.lx, cu.ly);
        tw.ray_o[0][i] = make_float4(r.o.x, r.o.y, r.o.z, r.t_max);
        tw.ray_d[0][i] = make_float4(r.d.x, r.d.y, r.d.z, r.time);
        tw.beta[0][i] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        tw.meta[0][i] = make_uint4(i, 1u, 0u, tw.textured);
        if (tw.textured) store_rd(tw.rd[0], i, camera_diff(cam, fx, fy, r, rp.diff_scale, cu.lx, cu.ly));
        tw.L[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

// Before level d: the next level's queue and the shadow queue start empty.
__global__ void k_tw_prep(TreeWave tw, uint32_t d) {
    tw.counters[(d + 1) & 1] = 0;
    tw.counters[TW_SHADOW] = 0;
    tw.counters[TW_EXT_HEAD] = 0;
    tw.counters[TW_SH_HEAD] = 0;
}

struct TwExtSrc {
    TreeWave tw;
    uint32_t b;
    BG_D Ray load(uint32_t i, int* skip) const {
        *skip = -1;
        return load_ray(tw.ray_o[b][i], tw.ray_d[b][i]);
    }
    BG_D void store(uint32_t i, int prim, float t) const { tw.hit[i] = make_int2(prim, __float_as_int(t)); }
};

template <int LAYOUT>
__global__ void __launch_bounds__(128, BG_MINBLOCKS) k_tw_extend(Scene sc, TreeWave tw, uint32_t d, uint32_t* err,
                                                                 int refill) {
    const uint32_t n = min(tw.counters[d & 1], tw.cap);
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&tw.ray_stats[0], (unsigned long long)n);
    TwExtSrc src{tw, d & 1u};
#if BG_SMEM_STACK
    __shared__ uint2 stack8[LAYOUT == 8 ? STACK8 * 128 : 1];
#else
    uint2* stack8 = nullptr;
#endif
    if (LAYOUT == 8) traverse_queue8<false>(sc, n, &tw.counters[TW_EXT_HEAD], src, err, refill, stack8);
    else traverse_queue<false>(sc, n, &tw.counters[TW_EXT_HEAD], src, err, refill);
}


struct TwShadowSrc {
    TreeWave tw;
    BG_D Ray load(uint32_t i, int* skip) const {
        const float4 o = tw.sh_o[i], dd = tw.sh_d[i];
        Ray r;
        r.o = f4xyz(o);
        r.t_max = o.w;
        r.d = f4xyz(dd);
        r.time = 0.0f;
        *skip = __float_as_int(dd.w);
        return r;
    }
    BG_D void store(uint32_t i, int prim, float) const {
        if (prim >= 0) return;
        const float4 c = tw.sh_c[i];
        add_L(tw, __float_as_uint(c.w), rgb(c.x, c.y, c.z));
    }
};

template <int LAYOUT>
__global__ void __launch_bounds__(128, BG_MINBLOCKS) k_tw_shadow(Scene sc, TreeWave tw, uint32_t* err, int refill) {
    const uint32_t n = min(tw.counters[TW_SHADOW], tw.sh_cap);
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&tw.ray_stats[1], (unsigned long long)n);
    TwShadowSrc src{tw};
#if BG_SMEM_STACK
    __shared__ uint2 stack8[LAYOUT == 8 ? STACK8 * 128 : 1];
#else
    uint2* stack8 = nullptr;
#endif
    if (LAYOUT == 8) traverse_queue8<true>(sc, n, &tw.counters[TW_SH_HEAD], src, err, refill, stack8);
    else traverse_queue<true>(sc, n, &tw.counters[TW_SH_HEAD], src, err, refill);
}

// Each sample's total into the film (SamplerIntegrator::render's checks in film_add).
__global__ void k_tw_final(RenderParams rp, FilmBuffers film, TreeWave tw, uint64_t item0, uint32_t n) {
    const uint64_t npix = (uint64_t)rp.width * rp.height;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 l = tw.L[i];
        film_add(film, pixel_of((uint32_t)((item0 + i) % npix), rp.width, rp.height, rp.pixel_tiles),
                 rgb(l.x, l.y, l.z));
    }
}

int launch_tree_wave(int kind, const Scene& sc, const Camera& cam, const RenderParams& rp, const TreeWave& tw,
                     uint64_t item0, uint32_t n, uint32_t* err, const LaunchShape& ls, cudaStream_t s) {
    int launches = 0;
    dim3 grid(ls.sms * ls.blocks_per_sm), block(128);
    k_tw_gen<<<grid, block, 0, s>>>(cam, rp, tw, item0, n);
    ++launches;
    const bool wide8 = sc.nodes8 != nullptr;
    for (uint32_t d = 0; d < rp.max_depth; ++d) {
        k_tw_prep<<<1, 1, 0, s>>>(tw, d);
        if (wide8) k_tw_extend<8><<<grid, block, 0, s>>>(sc, tw, d, err, ls.refill);
        else k_tw_extend<2><<<grid, block, 0, s>>>(sc, tw, d, err, ls.refill);
        if (kind == 1) launch_tw_shade_whitted(sc, rp, tw, d, item0, err, grid, block, s);
        else launch_tw_shade_direct(kind, sc, rp, tw, d, item0, err, grid, block, s);
        if (wide8) k_tw_shadow<8><<<grid, block, 0, s>>>(sc, tw, err, ls.refill);
        else k_tw_shadow<2><<<grid, block, 0, s>>>(sc, tw, err, ls.refill);
        launches += 4;
    }
    return launches;
}

void launch_tree_final(const RenderParams& rp, const FilmBuffers& film, const TreeWave& tw, uint64_t item0,
                       uint32_t n, const LaunchShape& ls, cudaStream_t s) {
    k_tw_final<<<ls.sms * 4, 256, 0, s>>>(rp, film, tw, item0, n);
}

}  // namespace bg

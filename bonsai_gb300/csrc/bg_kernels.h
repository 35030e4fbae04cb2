// bg_kernels.h - launch interface between the host driver (bg_api.cpp) and the kernels.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/bonsai_gpu.h"
#include "bg_device.h"

namespace bg {

struct RenderParams {
    uint32_t width, height, spp, max_depth, first_sample;
    float rr_threshold;
    uint64_t seed;
    float bmin[3], binv[3];  // scene bounds, for ray binning: cell = (p - bmin) * binv in [0,1)
    Camera cam;              // for the camera rays' differentials at the first hit (textures)
    float diff_scale;        // Ray::scale_differentials factor, 1 / sqrt(samples per pixel)
    StratParams strat;       // StratifiedSampler (dims = 0: the counter RNG alone)
    uint32_t pixel_tiles;    // wavefront camera rays in 8 x 4 pixel tiles (BG_TUNE_TILE_PIXELS)
};
// StratParams of a render's sampler options (sampler 0 independent, 1 stratified): nullptr when
// they are valid, otherwise why not.
inline const char* strat_params(uint32_t sampler, uint32_t spp, uint32_t nx, uint32_t ny, uint32_t dims,
                                uint32_t jitter, StratParams* sp) {
    *sp = StratParams{0u, 1u, 1u, 0u};
    if (sampler > 1) return "unknown sampler";
    if (sampler == 0) return nullptr;
    if (nx == 0 || ny == 0 || (uint64_t)nx * ny != spp)
        return "the stratified sampler needs spp == x_pixel_samples * y_pixel_samples";
    if (dims > 64) return "the stratified sampler accepts sampled_dimensions <= 64";
    if (jitter > 1) return "jitter_samples must be 0 or 1";
    *sp = StratParams{dims, nx, ny, jitter};
    return nullptr;
}
// RenderParams for a render call: camera and differential scale filled in.
inline RenderParams with_camera(RenderParams rp, const Camera& cam, uint32_t total_spp) {
    rp.cam = cam;
    rp.diff_scale = 1.0f / sqrtf((float)(total_spp ? total_spp : 1u));
    return rp;
}

struct FilmBuffers {
    double* sum;     // 3 per pixel
    double* sumsq;   // 3 per pixel
    uint32_t* count; // per pixel
    float* rgb;      // resolved, 3 per pixel
    float* pass;     // optional: sum of this pass's samples per pixel (3 floats), for per-pass variance
    unsigned long long* nan_count;
    uint32_t npix;
};

// Path-state arrays of one wavefront (capacity = number of path slots).
struct WaveBuffers {
    uint32_t capacity;
    float4* ray_o;      // o.xyz, t_max
    float4* ray_d;      // d.xyz, time
    int2* hit;          // prim, t bits
    uint32_t* pixel;
    uint32_t* sample;
    uint32_t* state;    // bounce | specular flag << 8 | pending flag << 9
    float4* beta;       // rgb, eta_scale
    float4* L;          // rgb
    float4* nee_beta;   // beta at the NEE vertex
    float4* pending;    // 2 per slot: contribution rgb, w = 1 if unoccluded
    uint32_t sh_capacity;  // shadow-queue entries: 2 * capacity, or capacity with BG_TUNE_SHADOW_QUEUE_HALF
    float4* sh_o;       // sh_capacity shadow rays: o.xyz, t_max
    float4* sh_d;       // d.xyz, skip prim (int bits)
    uint32_t* sh_ref;   // slot * 2 + kind
    uint32_t* queue[2];
    uint32_t* cls_queue;  // 5 * capacity: hits binned by material class (matte, plastic, conductor,
                          // dielectric) and misses, written by extend, read by the class's shade launch
    uint32_t* done;
    uint32_t* counters; // [0,1] queue sizes, [2] shadow count, [3] done count, [4] extend head,
                        // [5] shadow head, [6..10] class queue sizes, [11] guided queries
    unsigned long long* ray_stats;  // [0] closest-hit rays traced, [1] any-hit rays traced
    uint32_t* wavectl;              // graph replay: [0] wave index, [1] first sample (device side)
    uint32_t* scene_id;             // batch renders: scene of each path slot
    uint32_t* qsort;                // binned extension queue (BG_TUNE_SORT_RAYS)
    uint32_t* sort_hist;            // [0, 4096) bin counts, [4096, 8192) bin cursors
};

// One scene of a batch render (a device table of these): what a path of the scene needs.
struct SceneRender {
    Scene sc;
    Camera cam;
    RenderParams rp;
    FilmBuffers film;   // this scene's slice of the batch film
    uint64_t item0;     // first item (pixel x sample) of the scene in the batch's item space
};

// Guiding state of one wavefront (all null / zero for unguided renders).
//   record: every non-specular vertex whose continuation was sampled opens a training record
//           (query, wi, BSDF pdf, throughput before the vertex); the next shade of the path closes
//           it, splitting what arrived along wi into the emission found there (direct) and what
//           the path gathers after it (indirect); at the end of the path each record becomes a
//           training sample with weight f |cos| Li / p (luminance) of the selected target.
//   guided: the binning pass writes a network query for every matte / plastic / conductor hit,
//           the network infers their mixtures, and the shade kernel samples with the one-sample
//           mixture c * guide + (1 - c) * BSDF: as the second (direction-sampling) strategy of
//           estimate_direct (GW_NEE) and / or for the continuation (GW_CONT).
//   GW_CONT: the continuation is drawn from the continuation head's mixture (one-sample MIS with
//   the BSDF); GW_NEE: estimate_direct's second strategy is drawn from the next-event head's
//   mixture (otherwise either stays a BSDF sample).
enum : uint32_t { GW_RECORD = 1u, GW_GUIDED = 2u, GW_CONT = 4u, GW_NEE = 8u };
constexpr int GUIDE_MAXREC = 6;      // training records kept per path
constexpr int GUIDE_REC_F4 = 5;      // float4 per record
constexpr uint32_t DIM_GUIDE0 = 4096;  // guided sampling uniforms: 8 per bounce from here

struct GuideWave {
    uint32_t flags;
    uint32_t pool_cap;   // training samples the pool holds
    float keep_prob;     // probability that a path records training samples (all enter the pool)
    uint32_t cap;        // path slots the record / query buffers below hold (>= the wave's paths)
    float4 bmin, binv;   // position encoding: p_norm = (p - bmin) * binv
    float4* rec;         // GUIDE_MAXREC * GUIDE_REC_F4 * cap, [k][field][slot]
    // guided queries of material class c (matte, plastic, conductor) at c * cap + the path's
    // position in the class queue
    float4* query;       // 3 float4 per query (3 * cap queries)
    float* raw;          // mixture records of both heads, head-major (mix_head_stride)
    float4* pool;        // 4 float4 per training sample
    // the light sample of a recording path's last vertex as a next-event training sample (4 float4
    // per slot, two buffers by bounce parity), emitted once its shadow test has resolved
    float4* lrec;
    uint32_t* ctr;       // [0] positive-weight records, [1] pool appends (kept)
    const uint8_t* wpack;  // BF16 weight image
};

// Streams and events that let a bounce's material-class shade kernels run side by side: forked
// from the launching stream after binning and joined back before the shadow rays (also inside a
// stream capture, where they become parallel graph branches).
struct ShadeFork {
    cudaStream_t aux[4];
    cudaEvent_t fork, join[4];
};

struct LaunchShape {
    int sms;
    int block;
    int blocks_per_sm = 8;
    int refill = 32;
    int sort_rays = 0;
    int l2_persist = 0;  // BG_TUNE_L2_PERSIST (part of the captured graph's key)
    // BG_TUNE_TILE_PIXELS, on by default: production 1080p at 16 spp 169.4 ms against 174.1 ms in
    // scanline order (extension 104.8 against 108.7 ms), Whitted 443 against 460 ms
    int tile_pixels = 1;
    int shadow_half = 0;  // BG_TUNE_SHADOW_QUEUE_HALF
    const ShadeFork* fork = nullptr;  // BG_TUNE_CONCURRENT_SHADE: the context's shade streams
};

void launch_trace(const Scene& sc, bool ref_layout, bool any, const bg_ray* rays, size_t n, bg_hit* hits,
                  uint8_t* occluded, uint32_t* err, unsigned long long* counters, uint32_t* work_head,
                  const LaunchShape& ls, cudaStream_t s);
// Breadth-first wavefront of the Whitted / direct-lighting ray trees (bg_tree_wave.cu).  One wave
// = up to `nsamp` camera samples; level d of every sample's tree is one queue of tree nodes (depth
// d), ping-ponged between two buffers; light-sampling rays of a level go to one shadow queue.
// Contributions add into per-sample accumulators, which reach the film once the wave's trees are
// done.  counters: [0,1] level sizes, [2] shadow rays, [3] extension head, [4] shadow head,
// [5] overflow (a level or the shadow queue outgrew its capacity: the wave is redone smaller).
struct TreeWave {
    uint32_t cap, sh_cap, samp_cap;
    uint32_t textured;
    float4* ray_o[2];   // o.xyz, t_max
    float4* ray_d[2];   // d.xyz, time
    float4* beta[2];    // rgb
    uint4* meta[2];     // sample slot, node id, depth, has differentials
    float4* rd[2];      // 4 per node: rx origin, ry origin, rx direction, ry direction (textured scenes)
    int2* hit;          // closest hit of the current level's nodes
    float4* sh_o;       // shadow ray origin, t_max
    float4* sh_d;       // direction, prim to skip (int bits)
    float4* sh_c;       // contribution rgb, sample slot (uint bits)
    float4* L;          // per sample slot: radiance accumulated so far
    uint32_t* counters;
    unsigned long long* ray_stats;  // [0] closest-hit rays, [1] any-hit rays
};
// Traces and shades the trees of samples [item0, item0 + n) (item = sample * npix + pixel, as the
// path wavefront) into the wave's accumulators; returns the kernel launches.  kind as below.  The
// host then reads counters[5]: zero -> launch_tree_final adds the samples to the film; set -> the
// wave outgrew a queue and is rendered again in smaller waves (nothing reached the film).
int launch_tree_wave(int kind, const Scene& sc, const Camera& cam, const RenderParams& rp, const TreeWave& tw,
                     uint64_t item0, uint32_t n, uint32_t* err, const LaunchShape& ls, cudaStream_t s);
void launch_tree_final(const RenderParams& rp, const FilmBuffers& film, const TreeWave& tw, uint64_t item0,
                       uint32_t n, const LaunchShape& ls, cudaStream_t s);

// Whitted / direct-lighting integrators (bg_integrators.cu): kind 1 Whitted, 2 direct lighting with
// UniformSampleAll, 3 direct lighting with UniformSampleOne; layout 1 reference, 2 two-wide,
// 8 eight-wide.  Tree depth is limited to TREE_MAX_DEPTH (a specular ray tree's pending-ray
// stack holds at most max_depth + 1 entries).
constexpr uint32_t TREE_MAX_DEPTH = 30;
constexpr int TREE_STACK = (int)TREE_MAX_DEPTH + 2;
void launch_tree_integrator(int kind, bool ref_compat, int layout, const Scene& sc, const Camera& cam,
                            const RenderParams& rp, const FilmBuffers& film, uint32_t* err, const LaunchShape& ls,
                            cudaStream_t s);
void launch_megakernel(bool ref_compat, const Scene& sc, const Camera& cam, const RenderParams& rp,
                       const FilmBuffers& film, uint32_t* err, const LaunchShape& ls, cudaStream_t s);
// One wave of the PBRT wavefront: items [item0, item0 + nitems) of the pixel x sample space.
// Returns the number of kernels launched.  stage_events (optional): 4 events per bounce, recorded
// before extend, before shade, before shadow and before finalize.
// gw (optional): guiding state; guided waves write the network queries while binning and run the
// network inference before the material shades of every bounce.
int launch_wave(const Scene& sc, const Camera& cam, const RenderParams& rp, const FilmBuffers& film,
                const WaveBuffers& wb, uint64_t item0, uint32_t nitems, uint32_t* err, const LaunchShape& ls,
                cudaStream_t s, cudaEvent_t* stage_events, const GuideWave* gw = nullptr);
// The same stage chain with the wave index and first sample read from wb.wavectl, advanced by the
// chain itself: a static launch sequence that is captured once into a CUDA graph and replayed
// for every wave.  Returns the number of kernels in the chain.
int launch_wave_chain(const Scene& sc, const Camera& cam, const RenderParams& rp, const FilmBuffers& film,
                      const WaveBuffers& wb, uint64_t total, uint32_t* err, const LaunchShape& ls, cudaStream_t s);
// One wave of a batch render: items [item0, item0 + nitems) of the concatenated item spaces of
// `nscenes` scenes (tab, device); paths of all scenes share the queues of one set of launches
// (8-wide BVH layouts).  max_depth = the largest of the scenes'.  Returns the kernels launched.
// variants: bit 0 some scene is textured, bit 1 some scene holds an infinite light (the shade
// launches then take the variants that handle both per scene).
int launch_wave_batch(const SceneRender* tab, uint32_t nscenes, uint32_t max_depth, const WaveBuffers& wb,
                      uint64_t item0, uint32_t nitems, uint32_t* err, const LaunchShape& ls, cudaStream_t s,
                      uint32_t variants = 0);
void launch_resolve(const FilmBuffers& film, cudaStream_t s);
void launch_clear_film(const FilmBuffers& film, cudaStream_t s);

}  // namespace bg

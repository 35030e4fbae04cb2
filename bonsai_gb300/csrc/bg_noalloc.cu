// bg_noalloc.cu - bg_render_noalloc: the render entry point for callers that cannot allocate
// device memory.
//
// Some hosts cannot call cudaMalloc during a frame: a renderer plugin whose host application owns
// the device memory budget and forbids allocation outside load time, a process under a fixed
// memory reservation, or a frame loop that must never block in the allocator.  This entry point
// allocates nothing.  Its scratch memory (film moments, wavefront queues and path state,
// counters, the device error word) is the file-scope array g_scratch below, sized for at most
// BG_NOALLOC_MAX_PIXELS pixels and a wave of BG_NOALLOC_WAVE_PATHS paths.  Every GPU that loads
// the library holds this array until the process exits.
//
// The array's name is only a host-side stand-in in host code; the first call on each device (with
// that device current) resolves its device address with cudaGetSymbolAddress and caches it.  Make
// that first call before any stream capture.  All calls share the one array and it keeps the last
// call's contents, so each call clears what must start at zero; calls that overlap on the GPU
// (two streams, two host threads) race on the array and must be serialised by the caller.  A call
// is synchronous: it waits for its stream to finish the render and reads the device error word
// back before it returns.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/bonsai_gpu.h"
#include "bg_kernels.h"

namespace bg {

// Scene internals exposed by bg_api.cpp.
bool scene_device_view(const bg_scene* s, Scene* dev, uint32_t* kind, int* device);
void scene_set_error(const bg_scene* s, const std::string& msg);
Camera camera_for(const bg_camera& c);

namespace {

constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

constexpr size_t P = BG_NOALLOC_MAX_PIXELS;
constexpr size_t N = BG_NOALLOC_WAVE_PATHS;
// carve order: film, wave, counters
constexpr size_t OFF_SUM = 0;
constexpr size_t OFF_SUMSQ = OFF_SUM + align_up(P * 3 * sizeof(double));
constexpr size_t OFF_COUNT = OFF_SUMSQ + align_up(P * 3 * sizeof(double));
constexpr size_t OFF_NAN = OFF_COUNT + align_up(P * sizeof(uint32_t));
constexpr size_t OFF_ERR = OFF_NAN + align_up(sizeof(unsigned long long));
constexpr size_t OFF_COUNTERS = OFF_ERR + align_up(sizeof(uint32_t));
constexpr size_t OFF_RAYSTATS = OFF_COUNTERS + align_up(16 * sizeof(uint32_t));
constexpr size_t OFF_RAY_O = OFF_RAYSTATS + align_up(4 * sizeof(unsigned long long));
constexpr size_t OFF_RAY_D = OFF_RAY_O + align_up(N * sizeof(float4));
constexpr size_t OFF_HIT = OFF_RAY_D + align_up(N * sizeof(float4));
constexpr size_t OFF_PIXEL = OFF_HIT + align_up(N * sizeof(int2));
constexpr size_t OFF_SAMPLE = OFF_PIXEL + align_up(N * sizeof(uint32_t));
constexpr size_t OFF_STATE = OFF_SAMPLE + align_up(N * sizeof(uint32_t));
constexpr size_t OFF_BETA = OFF_STATE + align_up(N * sizeof(uint32_t));
constexpr size_t OFF_L = OFF_BETA + align_up(N * sizeof(float4));
constexpr size_t OFF_NEE = OFF_L + align_up(N * sizeof(float4));
constexpr size_t OFF_PENDING = OFF_NEE + align_up(N * sizeof(float4));
constexpr size_t OFF_SH_O = OFF_PENDING + align_up(2 * N * sizeof(float4));
constexpr size_t OFF_SH_D = OFF_SH_O + align_up(2 * N * sizeof(float4));
constexpr size_t OFF_SH_REF = OFF_SH_D + align_up(2 * N * sizeof(float4));
constexpr size_t OFF_Q0 = OFF_SH_REF + align_up(2 * N * sizeof(uint32_t));
constexpr size_t OFF_Q1 = OFF_Q0 + align_up(N * sizeof(uint32_t));
constexpr size_t OFF_CLS = OFF_Q1 + align_up(N * sizeof(uint32_t));
constexpr size_t OFF_DONE = OFF_CLS + align_up(5 * N * sizeof(uint32_t));
constexpr size_t SCRATCH_BYTES = OFF_DONE + align_up(N * sizeof(uint32_t));
static_assert(SCRATCH_BYTES == BG_NOALLOC_SCRATCH_BYTES, "keep BG_NOALLOC_SCRATCH_BYTES in step");

static __device__ __align__(256) unsigned char g_scratch[SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned char* g_scratch_dev[kMaxDevices] = {nullptr};

// Once per device, with that device current: the device address of g_scratch.
bg_status scratch_for_device(int device, unsigned char** out, std::string* why) {
    if (device < 0 || device >= kMaxDevices) {
        *why = "device ordinal out of range";
        return BG_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_dev[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) {
            *why = std::string("cudaGetSymbolAddress(g_scratch): ") + cudaGetErrorString(e);
            return e == cudaErrorNoKernelImageForDevice ? BG_ERR_NO_DEVICE : BG_ERR_CUDA;
        }
        g_scratch_dev[device] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_dev[device];
    return BG_OK;
}

}  // namespace
}  // namespace bg

extern "C" bg_status bg_render_noalloc(const bg_scene* scene, const bg_camera* cam, const bg_render_opts* o,
                                       float* d_rgb_out, void* cuda_stream) {
    using namespace bg;
    if (!scene || !cam || !o || !d_rgb_out) return BG_ERR_INVALID;
    Scene dev{};
    uint32_t kind = 0;
    int device = 0;
    if (!scene_device_view(scene, &dev, &kind, &device)) return BG_ERR_INVALID;
    auto reject = [&](bg_status st, const std::string& msg) {
        scene_set_error(scene, "bg_render_noalloc: " + msg);
        return st;
    };
    const uint64_t npix = (uint64_t)cam->width * cam->height;
    if (cam->width == 0 || cam->height == 0) return reject(BG_ERR_INVALID, "empty film");
    if (npix > BG_NOALLOC_MAX_PIXELS)
        return reject(BG_ERR_INVALID, std::to_string(cam->width) + "x" + std::to_string(cam->height) +
                                          " film exceeds the scratch limit of " +
                                          std::to_string(BG_NOALLOC_MAX_PIXELS) + " pixels");
    if (!(cam->lens_radius >= 0.0f) || !std::isfinite(cam->lens_radius))
        return reject(BG_ERR_INVALID, "lens_radius must be finite and >= 0");
    if (cam->lens_radius > 0.0f && (!(cam->focal_distance > 0.0f) || !std::isfinite(cam->focal_distance)))
        return reject(BG_ERR_INVALID, "a thin-lens camera needs a finite focal_distance > 0");
    if (!(cam->fov_deg > 0.0f && cam->fov_deg < 180.0f)) return reject(BG_ERR_INVALID, "fov out of range");
    if (o->mode > BG_MODE_PBRT) return reject(BG_ERR_INVALID, "unknown mode");
    if (o->mode == BG_MODE_REF_COMPAT && (kind == BG_BVH_WIDE || kind == BG_BVH_WIDE2))
        return reject(BG_ERR_INVALID, "REF_COMPAT rendering needs a BG_BVH_REFERENCE* scene layout");
    if (o->max_depth > 250) return reject(BG_ERR_INVALID, "max_depth must be <= 250");
    if (o->flags & (BG_RENDER_ACCUMULATE | BG_RENDER_STAGE_TIMING | BG_RENDER_GRAPH))
        return reject(BG_ERR_UNSUPPORTED, "accumulate / stage timing / graph flags need bg_render");
    if (o->integrator != BG_INTEGRATOR_PATH)
        return reject(BG_ERR_UNSUPPORTED, "the Whitted and direct-lighting integrators need bg_render");
    StratParams strat;
    if (const char* why = strat_params(o->sampler, o->spp, o->x_pixel_samples, o->y_pixel_samples,
                                       o->sampled_dimensions, o->jitter_samples, &strat))
        return reject(BG_ERR_INVALID, why);

    int prev = -1;
    cudaGetDevice(&prev);
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return reject(BG_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    auto finish = [&](bg_status st) {
        if (prev >= 0 && prev != device) cudaSetDevice(prev);
        return st;
    };
    unsigned char* base = nullptr;
    std::string why;
    bg_status st = scratch_for_device(device, &base, &why);
    if (st != BG_OK) return finish(reject(st, why));
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);

    FilmBuffers film{};
    film.sum = reinterpret_cast<double*>(base + OFF_SUM);
    film.sumsq = reinterpret_cast<double*>(base + OFF_SUMSQ);
    film.count = reinterpret_cast<uint32_t*>(base + OFF_COUNT);
    film.nan_count = reinterpret_cast<unsigned long long*>(base + OFF_NAN);
    film.rgb = d_rgb_out;
    film.npix = (uint32_t)npix;
    uint32_t* d_err = reinterpret_cast<uint32_t*>(base + OFF_ERR);
    WaveBuffers w{};
    w.capacity = (uint32_t)N;
    w.sh_capacity = 2 * (uint32_t)N;
    w.ray_o = reinterpret_cast<float4*>(base + OFF_RAY_O);
    w.ray_d = reinterpret_cast<float4*>(base + OFF_RAY_D);
    w.hit = reinterpret_cast<int2*>(base + OFF_HIT);
    w.pixel = reinterpret_cast<uint32_t*>(base + OFF_PIXEL);
    w.sample = reinterpret_cast<uint32_t*>(base + OFF_SAMPLE);
    w.state = reinterpret_cast<uint32_t*>(base + OFF_STATE);
    w.beta = reinterpret_cast<float4*>(base + OFF_BETA);
    w.L = reinterpret_cast<float4*>(base + OFF_L);
    w.nee_beta = reinterpret_cast<float4*>(base + OFF_NEE);
    w.pending = reinterpret_cast<float4*>(base + OFF_PENDING);
    w.sh_o = reinterpret_cast<float4*>(base + OFF_SH_O);
    w.sh_d = reinterpret_cast<float4*>(base + OFF_SH_D);
    w.sh_ref = reinterpret_cast<uint32_t*>(base + OFF_SH_REF);
    w.queue[0] = reinterpret_cast<uint32_t*>(base + OFF_Q0);
    w.queue[1] = reinterpret_cast<uint32_t*>(base + OFF_Q1);
    w.cls_queue = reinterpret_cast<uint32_t*>(base + OFF_CLS);
    w.done = reinterpret_cast<uint32_t*>(base + OFF_DONE);
    w.counters = reinterpret_cast<uint32_t*>(base + OFF_COUNTERS);
    w.ray_stats = reinterpret_cast<unsigned long long*>(base + OFF_RAYSTATS);

    // the array keeps the previous call's contents: zero what accumulates
    const struct {
        void* p;
        size_t bytes;
        const char* what;
    } clears[] = {{film.sum, npix * 3 * sizeof(double), "film sums"},
                  {film.sumsq, npix * 3 * sizeof(double), "film squared sums"},
                  {film.count, npix * sizeof(uint32_t), "film sample counts"},
                  {film.nan_count, sizeof(unsigned long long), "film NaN count"},
                  {d_err, sizeof(uint32_t), "error word"},
                  {w.counters, 16 * sizeof(uint32_t), "wave counters"},
                  {w.ray_stats, 4 * sizeof(unsigned long long), "ray statistics"}};
    for (const auto& c : clears) {
        e = cudaMemsetAsync(c.p, 0, c.bytes, s);
        if (e != cudaSuccess)
            return finish(reject(BG_ERR_CUDA, std::string("clearing the ") + c.what + ": " + cudaGetErrorString(e)));
    }

    int dev_sms = 0;
    e = cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess || dev_sms <= 0)
        return finish(reject(BG_ERR_CUDA, std::string("multiprocessor count: ") + cudaGetErrorString(e)));
    // fixed launch shape: bg_render's tuned shape and BG_TUNE_* settings belong to a bg_ctx, which
    // this entry point does not take
    LaunchShape shape{dev_sms, 128, 8, 32};
    Camera dc = camera_for(*cam);
    RenderParams rp{cam->width, cam->height, o->spp, o->max_depth, o->first_sample, o->rr_threshold, o->seed};
    rp = with_camera(rp, dc, o->spp);
    rp.strat = strat;
    rp.pixel_tiles = 1;  // camera rays in 8 x 4 pixel tiles, bg_render's default order
    const uint64_t total = npix * o->spp;
    if (total > 0) {
        if (o->mode == BG_MODE_PBRT && (kind == BG_BVH_WIDE || kind == BG_BVH_WIDE2)) {
            for (uint64_t item0 = 0; item0 < total; item0 += N) {
                uint32_t nitems = (uint32_t)((total - item0) < N ? (total - item0) : N);
                launch_wave(dev, dc, rp, film, w, item0, nitems, d_err, shape, s, nullptr);
            }
        } else {
            launch_megakernel(o->mode == BG_MODE_REF_COMPAT, dev, dc, rp, film, d_err, shape, s);
        }
    }
    launch_resolve(film, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return finish(reject(BG_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e)));
    uint32_t word = 0;
    e = cudaMemcpyAsync(&word, d_err, sizeof(word), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return finish(reject(BG_ERR_CUDA, std::string("sync: ") + cudaGetErrorString(e)));
    if (word) return finish(reject(BG_ERR_DEVICE, "device error word " + std::to_string(word)));
    return finish(BG_OK);
}

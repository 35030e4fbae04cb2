// bg_guide_api.cpp - C ABI of the guiding network and the progressive guided render.
//
// bg_render_guided renders opts->spp samples in passes of max(1, pass_paths / pixels) spp; the network's warm-up count, fallback decision
// and variance estimates carry over between calls, so a long render can be issued in chunks.  Per
// pass: the wavefront renders the image (guided passes write a network query for every matte /
// plastic / conductor hit while binning and infer the two mixtures of each before shading, where
// the continuation head proposes the continuation and the next-event head the second strategy of
// estimate_direct); paths chosen with a keep probability (set from the previous pass's record
// count) write training records, which land in a pool of samples_per_pass samples; one reduction
// estimates the pass's relative variance against the mean of the earlier passes; then the pool is
// consumed in batch_size Adam steps.  One host synchronisation per pass reads the counters that
// steer the next pass (keep probability, fallback decision).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/bonsai_gpu.h"
#include "bg_guide_kernels.h"
#include "bg_guide_layout.h"
#include "bg_internal.h"

using namespace bgi;

struct bg_guide {
    bg_ctx* ctx = nullptr;
    bg_guide_opts o{};
    float* params = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    float* grad = nullptr;
    float* partial = nullptr;   // per-CTA gradient slices of one batch (kept zero in unused rows)
    uint32_t partial_blocks = 0;
    uint8_t* wpack = nullptr;
    uint32_t* step = nullptr;   // Adam step counter
    uint32_t* ctr = nullptr;    // [0] positive-weight records, [1] pool appends
    float* stats = nullptr;     // [0] loss, [1] samples with weight > 0
    double* relvar = nullptr;   // [0] sum of relative squared deviations, [1] terms
    float* wsum = nullptr;      // two per batch of the pool (one per head)
    float4* pool = nullptr;
    uint32_t pool_cap = 0;
    float* pass = nullptr;      // this pass's sample per pixel
    size_t pass_pix = 0;
    float4* rec = nullptr;
    float4* lrec = nullptr;
    float4* query = nullptr;
    float* raw = nullptr;
    uint32_t wcap = 0;
    std::vector<void*> allocs, wave_allocs, pass_allocs;
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};  // pass, training and call timing
    // progressive state, carried across bg_render_guided calls
    uint64_t passes_total = 0;    // passes rendered with this network (warm-up counts these)
    bool fallback = false;        // plain BSDF sampling took over
    float keep = 1.0f;            // pool keep probability for the next pass
    double rv_plain_sum = 0, ms_plain_sum = 0;
    uint32_t n_plain = 0;
    // guided passes in the running estimate; the fallback is decided only once 2 kWindow guided
    // passes have trained the network (an early, half-trained guide is not the one that renders)
    static constexpr uint32_t kWindow = 32;
    double rv_guided[kWindow] = {}, ms_guided[kWindow] = {};
    uint32_t n_guided = 0;
    uint32_t pool_n = 0;          // samples in the pool after the last pass
    uint64_t epochs_done = 0;     // shuffling seed
};

namespace {

bg_guide_opts default_opts() {
    bg_guide_opts o{};
    o.learning_rate = 1e-3f;
    o.beta1 = 0.9f;
    o.beta2 = 0.999f;
    o.eps = 1e-8f;
    o.alpha = 0.5f;
    o.batch_size = 16384;
    o.samples_per_pass = 1u << 18;
    o.warmup_passes = 4;
    o.flags = 0;
    o.seed = 0;
    o.pass_paths = 1u << 22;
    o.epochs = 1;
    return o;
}

void free_guide_device(bg_guide* g) {
    if (!g->ctx) return;
    dfree_all(g->ctx, g->allocs);
    dfree_all(g->ctx, g->wave_allocs);
    dfree_all(g->ctx, g->pass_allocs);
    for (auto& e : g->ev)
        if (e) {
            cudaEventDestroy(e);
            e = nullptr;
        }
}

// He-uniform hidden layers, a 0.1-scaled output layer (near-uniform initial mixture), zero
// biases and zero padding.
std::vector<float> init_params(uint64_t seed) {
    std::vector<float> p(bg::GUIDE_PARAMS, 0.0f);
    std::mt19937_64 rng(seed ^ 0x9E3779B97F4A7C15ull);
    std::uniform_real_distribution<float> u(-1.0f, 1.0f);
    for (int l = 0; l < bg::GUIDE_LAYERS; ++l) {
        const int fan_in = l == 0 ? bg::GUIDE_IN_USED : bg::GUIDE_HID;
        float bound = std::sqrt(6.0f / (float)fan_in);
        if (l == bg::GUIDE_LAYERS - 1) bound *= 0.1f;
        for (int r = 0; r < bg::guide_used_rows(l); ++r)
            for (int c = 0; c < fan_in; ++c) p[bg::guide_param_off(l) + r * bg::GUIDE_K + c] = bound * u(rng);
    }
    return p;
}

// Padding entries the network never uses must stay zero (they would otherwise be trained by
// nothing and read by nothing, but keep the layout canonical).
bool padding_is_zero(const float* p) {
    for (int l = 0; l < bg::GUIDE_LAYERS; ++l) {
        const int used_in = l == 0 ? bg::GUIDE_IN_USED + 1 : bg::GUIDE_HID + 1;
        for (int r = 0; r < bg::guide_rows(l); ++r)
            for (int c = 0; c < bg::GUIDE_K; ++c)
                if ((r >= bg::guide_used_rows(l) || c >= used_in) && p[bg::guide_param_off(l) + r * bg::GUIDE_K + c] != 0.0f)
                    return false;
    }
    return true;
}

bg_status upload_params(bg_guide* g, const float* host) {
    bg_ctx* ctx = g->ctx;
    CK(cudaMemcpyAsync(g->params, host, bg::GUIDE_PARAMS * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(g->m, 0, bg::GUIDE_PARAMS * sizeof(float), ctx->stream));
    CK(cudaMemsetAsync(g->v, 0, bg::GUIDE_PARAMS * sizeof(float), ctx->stream));
    CK(cudaMemsetAsync(g->grad, 0, bg::GUIDE_PARAMS * sizeof(float), ctx->stream));
    CK(cudaMemsetAsync(g->step, 0, sizeof(uint32_t), ctx->stream));
    CK(cudaMemsetAsync(g->wpack, 0, bg::GUIDE_WPACK_BYTES, ctx->stream));
    bg::launch_guide_pack(g->params, g->wpack, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->stream));  // host is a caller buffer
    return BG_OK;
}

bg_status guide_error(bg_ctx* ctx) {
    uint32_t word = 0;
    bg_status st = check_device_error(ctx, &word);
    if (st != BG_OK && (word & bg::ERR_GUIDE_TIMEOUT))
        return fail(ctx, BG_ERR_TIMEOUT, "a tensor-core wait of the guiding network timed out");
    return st;
}

bg_status ensure_guide_wave(bg_guide* g, uint32_t cap) {
    if (g->wcap >= cap && g->rec) return BG_OK;
    bg_ctx* ctx = g->ctx;
    CK(cudaStreamSynchronize(ctx->stream));
    dfree_all(ctx, g->wave_allocs);
    g->wcap = 0;
    void* p;
    bg_status st;
    const size_t n = cap;
    if ((st = dalloc(ctx, (size_t)bg::GUIDE_MAXREC * bg::GUIDE_REC_F4 * n * sizeof(float4), &p, &g->wave_allocs)) != BG_OK)
        return st;
    g->rec = (float4*)p;
    // light-sample records of the recording paths' last vertices, two buffers by bounce parity
    if ((st = dalloc(ctx, 2 * 4 * n * sizeof(float4), &p, &g->wave_allocs)) != BG_OK) return st;
    g->lrec = (float4*)p;
    // queries and mixtures of the three guidable material classes, at class * cap + queue position
    if ((st = dalloc(ctx, 3 * 3 * n * sizeof(float4), &p, &g->wave_allocs)) != BG_OK) return st;
    g->query = (float4*)p;
    if ((st = dalloc(ctx, 3 * n * bg::GUIDE_MIX_STRIDE * sizeof(float), &p, &g->wave_allocs)) != BG_OK) return st;
    g->raw = (float*)p;
    g->wcap = cap;
    return BG_OK;
}

bg_status ensure_pass(bg_guide* g, size_t npix) {
    if (g->pass_pix == npix && g->pass) return BG_OK;
    bg_ctx* ctx = g->ctx;
    CK(cudaStreamSynchronize(ctx->stream));
    dfree_all(ctx, g->pass_allocs);
    void* p;
    bg_status st = dalloc(ctx, npix * 3 * sizeof(float), &p, &g->pass_allocs);
    if (st != BG_OK) return st;
    g->pass = (float*)p;
    g->pass_pix = npix;
    return BG_OK;
}

// Uploads n host samples into a temporary device buffer owned by `tmp`.
bg_status upload_samples(bg_guide* g, const float* samples, size_t n, float4** d, std::vector<void*>* tmp) {
    bg_ctx* ctx = g->ctx;
    void* p;
    bg_status st = dalloc(ctx, n * bg::GUIDE_SAMPLE_F4 * sizeof(float4), &p, tmp);
    if (st != BG_OK) return st;
    CK(cudaMemcpyAsync(p, samples, n * bg::GUIDE_SAMPLE_F4 * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream));
    *d = (float4*)p;
    return BG_OK;
}

uint32_t gcd32(uint32_t a, uint32_t b) {
    while (b) {
        uint32_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

// A pseudo-random visiting order of n pool entries for one epoch (multiplier coprime to n).
bg::PoolOrder pool_order(uint32_t n, uint64_t epoch) {
    bg::PoolOrder o{n, 1u, 0u, 0u};
    if (n < 2) return o;
    uint64_t h = (epoch + 1) * 0x9E3779B97F4A7C15ull;
    uint32_t mul = (uint32_t)(h >> 33) % n;
    while (mul < 2 || gcd32(mul, n) != 1) mul = (mul + 1) % n;
    o.perm_mul = mul;
    o.perm_add = (uint32_t)(h & 0xFFFFFFFFu) % n;
    return o;
}

// `epochs` passes over n samples in shuffled batches -> Adam steps (all asynchronous).  Returns the
// number of steps.
int train_batches(bg_guide* g, const float4* samples, uint32_t n, uint32_t epochs, uint64_t* epoch_counter) {
    bg_ctx* ctx = g->ctx;
    const uint32_t B = g->o.batch_size;
    const uint32_t nb = (n + B - 1) / B;
    cudaMemsetAsync(g->stats, 0, 2 * sizeof(float), ctx->stream);
    bg::GuideAdam h{g->o.learning_rate, g->o.beta1, g->o.beta2, g->o.eps};
    for (uint32_t e = 0; e < epochs; ++e) {
        bg::PoolOrder order = pool_order(n, (*epoch_counter)++);
        bg::launch_guide_wsum(samples, order, B, g->wsum, ctx->stream);
        for (uint32_t b = 0; b < nb; ++b) {
            bg::GuideTrainArgs a{};
            a.wpack = g->wpack;
            a.samples = samples;
            a.order = order;
            a.base = b * B;
            a.n = std::min(B, n - b * B);
            a.wsum = g->wsum + 2 * b;
            a.alpha = g->o.alpha;
            a.partial = g->partial;
            a.grad = g->grad;
            a.stats = g->stats;
            a.step = g->step;
            a.err = ctx->d_err;
            bg::launch_guide_train(a, ctx->stream);
            bg::launch_guide_adam(g->params, g->m, g->v, g->grad, g->wpack, g->step, h, ctx->stream);
        }
    }
    return (int)(nb * epochs);
}

}  // namespace

namespace bgi {
// Called by bg_destroy: guides outliving their context keep only host state.
void guide_orphan_all(bg_ctx* ctx) {
    for (bg_guide* g : ctx->guides) {
        free_guide_device(g);
        g->ctx = nullptr;
    }
    ctx->guides.clear();
}
}  // namespace bgi

extern "C" {

bg_status bg_guide_create(bg_ctx* ctx, const bg_guide_opts* opts, bg_guide** out) {
    if (!ctx || !out) return BG_ERR_INVALID;
    *out = nullptr;
    bg_guide_opts o = opts ? *opts : default_opts();
    if (o.batch_size == 0 || o.batch_size % 128 != 0) return fail(ctx, BG_ERR_INVALID, "batch_size must be a positive multiple of 128");
    if (o.samples_per_pass < 128 || o.samples_per_pass > (1u << 24))
        return fail(ctx, BG_ERR_INVALID, "samples_per_pass must be in [128, 2^24]");
    if (o.pass_paths == 0) o.pass_paths = 1u << 22;
    if (o.epochs == 0) o.epochs = 1;
    if (o.epochs > 64) return fail(ctx, BG_ERR_INVALID, "epochs must be <= 64");
    if (!(o.learning_rate > 0.0f) || !(o.alpha >= 0.0f && o.alpha <= 1.0f) || !(o.beta1 >= 0.0f && o.beta1 < 1.0f) ||
        !(o.beta2 >= 0.0f && o.beta2 < 1.0f) || !(o.eps > 0.0f))
        return fail(ctx, BG_ERR_INVALID, "bad optimiser settings");
    CK(cudaSetDevice(ctx->device));
    bg_guide* g = new bg_guide();
    g->ctx = ctx;
    g->o = o;
    auto bail = [&](bg_status s) {
        free_guide_device(g);
        delete g;
        return s;
    };
    void* p;
    bg_status st;
    const size_t pb = bg::GUIDE_PARAMS * sizeof(float);
    if ((st = dalloc(ctx, 4 * pb, &p, &g->allocs)) != BG_OK) return bail(st);
    g->params = (float*)p;
    g->m = g->params + bg::GUIDE_PARAMS;
    g->v = g->m + bg::GUIDE_PARAMS;
    g->grad = g->v + bg::GUIDE_PARAMS;
    if ((st = dalloc(ctx, bg::GUIDE_WPACK_BYTES, &p, &g->allocs)) != BG_OK) return bail(st);
    g->wpack = (uint8_t*)p;
    if ((st = dalloc(ctx, 64, &p, &g->allocs)) != BG_OK) return bail(st);
    g->step = (uint32_t*)p;
    g->ctr = (uint32_t*)((char*)p + 4);
    g->stats = (float*)((char*)p + 16);
    g->relvar = (double*)((char*)p + 32);
    g->pool_cap = o.samples_per_pass;
    if ((st = dalloc(ctx, (size_t)g->pool_cap * bg::GUIDE_SAMPLE_F4 * sizeof(float4), &p, &g->allocs)) != BG_OK)
        return bail(st);
    g->pool = (float4*)p;
    if ((st = dalloc(ctx, ((size_t)g->pool_cap / 128 + 1) * 2 * sizeof(float), &p, &g->allocs)) != BG_OK) return bail(st);
    g->wsum = (float*)p;
    g->partial_blocks = o.batch_size / 128;
    if ((st = dalloc(ctx, (size_t)g->partial_blocks * bg::GUIDE_PARAMS * sizeof(float), &p, &g->allocs)) != BG_OK)
        return bail(st);
    g->partial = (float*)p;
    if (cudaMemsetAsync(g->partial, 0, (size_t)g->partial_blocks * bg::GUIDE_PARAMS * sizeof(float), ctx->stream) !=
        cudaSuccess)
        return bail(BG_ERR_CUDA);
    for (auto& e : g->ev)
        if (cudaEventCreate(&e) != cudaSuccess) return bail(fail(ctx, BG_ERR_CUDA, "cudaEventCreate"));
    if (cudaMemsetAsync(g->step, 0, 64, ctx->stream) != cudaSuccess) return bail(BG_ERR_CUDA);
    std::vector<float> init = init_params(o.seed);
    if ((st = upload_params(g, init.data())) != BG_OK) return bail(st);
    ctx->guides.insert(g);
    *out = g;
    return BG_OK;
}

void bg_guide_destroy(bg_guide* g) {
    if (!g) return;
    if (g->ctx) {
        cudaSetDevice(g->ctx->device);
        cudaStreamSynchronize(g->ctx->stream);
        g->ctx->guides.erase(g);
        free_guide_device(g);
    }
    delete g;
}

bg_status bg_guide_set_wait_limit(bg_guide* g, uint64_t cycles) {
    if (!g || !g->ctx) return BG_ERR_INVALID;
    bg_ctx* ctx = g->ctx;
    CK(cudaSetDevice(ctx->device));
    CK(bg::set_guide_wait_limit(cycles, ctx->stream));
    return BG_OK;
}

bg_status bg_guide_get_params(bg_guide* g, float* params) {
    if (!g || !g->ctx || !params) return BG_ERR_INVALID;
    bg_ctx* ctx = g->ctx;
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync(params, g->params, bg::GUIDE_PARAMS * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return BG_OK;
}

bg_status bg_guide_set_params(bg_guide* g, const float* params) {
    if (!g || !g->ctx || !params) return BG_ERR_INVALID;
    bg_ctx* ctx = g->ctx;
    for (uint32_t i = 0; i < bg::GUIDE_PARAMS; ++i)
        if (!std::isfinite(params[i])) return fail(ctx, BG_ERR_INVALID, "non-finite parameter");
    if (!padding_is_zero(params)) return fail(ctx, BG_ERR_INVALID, "padding entries of the parameter layout must be zero");
    CK(cudaSetDevice(ctx->device));
    return upload_params(g, params);
}

bg_status bg_guide_forward(bg_guide* g, const float* queries, size_t n, float* out) {
    if (!g || !g->ctx || (n && (!queries || !out))) return BG_ERR_INVALID;
    bg_ctx* ctx = g->ctx;
    if (n == 0) return BG_OK;
    if (n >= (1u << 28)) return fail(ctx, BG_ERR_INVALID, "too many queries");
    CK(cudaSetDevice(ctx->device));
    std::vector<float4> q(3 * n);
    for (size_t i = 0; i < n; ++i) {
        const float* s = queries + 9 * i;
        q[3 * i] = make_float4(s[0], s[1], s[2], s[3]);
        q[3 * i + 1] = make_float4(s[4], s[5], s[6], s[7]);
        q[3 * i + 2] = make_float4(s[8], 0.0f, 0.0f, 0.0f);
    }
    std::vector<void*> tmp;
    void *dq = nullptr, *dr = nullptr;
    bg_status st = dalloc(ctx, q.size() * sizeof(float4), &dq, &tmp);
    if (st == BG_OK) st = dalloc(ctx, n * bg::GUIDE_RAW_STRIDE * sizeof(float), &dr, &tmp);
    std::vector<float> raw;
    if (st == BG_OK) {
        cudaMemcpyAsync(dq, q.data(), q.size() * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream);
        bg::launch_guide_infer(g->wpack, (const float4*)dq, nullptr, 1, (uint32_t)n, (float*)dr, false, ctx->d_err,
                               ctx->shape.sms, ctx->stream);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) st = cuda_fail(ctx, e, "k_guide_infer");
    }
    if (st == BG_OK) st = guide_error(ctx);
    if (st == BG_OK) {
        raw.resize(n * bg::GUIDE_RAW_STRIDE);
        cudaError_t e = cudaMemcpyAsync(raw.data(), dr, raw.size() * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) st = cuda_fail(ctx, e, "cudaMemcpyAsync");
    }
    cudaStreamSynchronize(ctx->stream);
    dfree_all(ctx, tmp);
    if (st != BG_OK) return st;
    for (size_t i = 0; i < n; ++i) std::memcpy(out + bg::GUIDE_OUT * i, raw.data() + bg::GUIDE_RAW_STRIDE * i, bg::GUIDE_OUT * sizeof(float));
    return BG_OK;
}

bg_status bg_guide_gradient(bg_guide* g, const float* samples, size_t n, float* grad, float* loss) {
    if (!g || !g->ctx || !samples || n == 0 || !grad) return BG_ERR_INVALID;
    bg_ctx* ctx = g->ctx;
    if (n >= (1u << 24)) return fail(ctx, BG_ERR_INVALID, "too many samples");
    CK(cudaSetDevice(ctx->device));
    std::vector<void*> tmp;
    float4* ds = nullptr;
    bg_status st = upload_samples(g, samples, n, &ds, &tmp);
    if (st == BG_OK) {
        cudaMemsetAsync(g->grad, 0, bg::GUIDE_PARAMS * sizeof(float), ctx->stream);
        cudaMemsetAsync(g->stats, 0, 2 * sizeof(float), ctx->stream);
        const bg::PoolOrder order{(uint32_t)n, 1u, 0u, 0u};
        bg::launch_guide_wsum(ds, order, (uint32_t)n, g->wsum, ctx->stream);
        // in chunks of the partial buffer's batch; every chunk's gradient adds into g->grad
        const uint32_t chunk = g->partial_blocks * 128;
        for (uint32_t base = 0; base < (uint32_t)n; base += chunk) {
            bg::GuideTrainArgs a{};
            a.wpack = g->wpack;
            a.samples = ds;
            a.order = order;
            a.base = base;
            a.n = std::min<uint32_t>(chunk, (uint32_t)n - base);
            a.wsum = g->wsum;
            a.alpha = g->o.alpha;
            a.partial = g->partial;
            a.grad = g->grad;
            a.stats = g->stats;
            a.step = nullptr;
            a.err = ctx->d_err;
            bg::launch_guide_train(a, ctx->stream);
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) st = cuda_fail(ctx, e, "k_guide_train");
    }
    if (st == BG_OK) st = guide_error(ctx);
    float stats[2] = {0, 0};
    if (st == BG_OK) {
        cudaError_t e = cudaMemcpyAsync(grad, g->grad, bg::GUIDE_PARAMS * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(stats, g->stats, sizeof(stats), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(g->grad, 0, bg::GUIDE_PARAMS * sizeof(float), ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) st = cuda_fail(ctx, e, "gradient readback");
    }
    cudaStreamSynchronize(ctx->stream);
    dfree_all(ctx, tmp);
    if (st == BG_OK && loss) *loss = stats[0];
    return st;
}

bg_status bg_guide_train(bg_guide* g, const float* samples, size_t n, float* loss) {
    if (!g || !g->ctx || (n && !samples)) return BG_ERR_INVALID;
    bg_ctx* ctx = g->ctx;
    if (n == 0) return BG_OK;
    if (n >= (1u << 24)) return fail(ctx, BG_ERR_INVALID, "too many samples");
    if ((n + g->o.batch_size - 1) / g->o.batch_size > (size_t)g->pool_cap / 128 + 1)
        return fail(ctx, BG_ERR_INVALID, "too many batches for this network's batch-sum buffer");
    CK(cudaSetDevice(ctx->device));
    std::vector<void*> tmp;
    float4* ds = nullptr;
    bg_status st = upload_samples(g, samples, n, &ds, &tmp);
    int nb = 0;
    if (st == BG_OK) {
        nb = train_batches(g, ds, (uint32_t)n, 1, &g->epochs_done);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) st = cuda_fail(ctx, e, "guide training");
    }
    if (st == BG_OK) st = guide_error(ctx);
    float stats[2] = {0, 0};
    if (st == BG_OK) {
        cudaError_t e = cudaMemcpyAsync(stats, g->stats, sizeof(stats), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) st = cuda_fail(ctx, e, "loss readback");
    }
    cudaStreamSynchronize(ctx->stream);
    dfree_all(ctx, tmp);
    if (st == BG_OK && loss) *loss = nb ? stats[0] / (float)nb : 0.0f;
    return st;
}

bg_status bg_guide_pool(bg_guide* g, float* out, size_t max_n, size_t* n_out) {
    if (!g || !g->ctx || (max_n && !out)) return BG_ERR_INVALID;
    bg_ctx* ctx = g->ctx;
    const size_t n = std::min<size_t>(max_n, g->pool_n);
    CK(cudaSetDevice(ctx->device));
    if (n) {
        CK(cudaMemcpyAsync(out, g->pool, n * bg::GUIDE_SAMPLE_F4 * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    if (n_out) *n_out = n;
    return BG_OK;
}

bg_status bg_guide_time(bg_guide* g, const float* samples, size_t n, const float* queries, size_t nq, uint32_t reps,
                        double* train_step_ms, double* infer_ms) {
    if (!g || !g->ctx || !samples || !queries || n == 0 || nq == 0 || reps == 0) return BG_ERR_INVALID;
    bg_ctx* ctx = g->ctx;
    if (n >= (1u << 24) || nq >= (1u << 28)) return fail(ctx, BG_ERR_INVALID, "too many samples or queries");
    CK(cudaSetDevice(ctx->device));
    std::vector<void*> tmp;
    float4* ds = nullptr;
    bg_status st = upload_samples(g, samples, n, &ds, &tmp);
    std::vector<float4> q(3 * nq);
    for (size_t i = 0; i < nq; ++i) {
        const float* a = queries + 9 * i;
        q[3 * i] = make_float4(a[0], a[1], a[2], a[3]);
        q[3 * i + 1] = make_float4(a[4], a[5], a[6], a[7]);
        q[3 * i + 2] = make_float4(a[8], 0.0f, 0.0f, 0.0f);
    }
    void *dq = nullptr, *dout = nullptr;
    if (st == BG_OK) st = dalloc(ctx, q.size() * sizeof(float4), &dq, &tmp);
    if (st == BG_OK) st = dalloc(ctx, nq * bg::GUIDE_MIX_STRIDE * sizeof(float), &dout, &tmp);
    float t_train = 0.0f, t_infer = 0.0f;
    if (st == BG_OK) {
        cudaMemcpyAsync(dq, q.data(), q.size() * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream);
        const uint32_t nb = (uint32_t)std::min<size_t>(n, g->o.batch_size);
        const bg::PoolOrder order{nb, 1u, 0u, 0u};
        bg::GuideAdam h{g->o.learning_rate, g->o.beta1, g->o.beta2, g->o.eps};
        bg::launch_guide_wsum(ds, order, nb, g->wsum, ctx->stream);
        auto step = [&]() {
            bg::GuideTrainArgs a{};
            a.wpack = g->wpack;
            a.samples = ds;
            a.order = order;
            a.base = 0;
            a.n = nb;
            a.wsum = g->wsum;
            a.alpha = g->o.alpha;
            a.partial = g->partial;
            a.grad = g->grad;
            a.stats = g->stats;
            a.step = g->step;
            a.err = ctx->d_err;
            bg::launch_guide_train(a, ctx->stream);
            bg::launch_guide_adam(g->params, g->m, g->v, g->grad, g->wpack, g->step, h, ctx->stream);
        };
        auto infer = [&]() {
            bg::launch_guide_infer(g->wpack, (const float4*)dq, nullptr, 1, (uint32_t)nq, (float*)dout, true, ctx->d_err,
                                   ctx->shape.sms, ctx->stream);
        };
        step();
        infer();
        cudaEventRecord(g->ev[0], ctx->stream);
        for (uint32_t r = 0; r < reps; ++r) step();
        cudaEventRecord(g->ev[1], ctx->stream);
        for (uint32_t r = 0; r < reps; ++r) infer();
        cudaEventRecord(g->ev[2], ctx->stream);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) st = cuda_fail(ctx, e, "guide timing");
    }
    if (st == BG_OK) st = guide_error(ctx);
    if (st == BG_OK) {
        cudaEventElapsedTime(&t_train, g->ev[0], g->ev[1]);
        cudaEventElapsedTime(&t_infer, g->ev[1], g->ev[2]);
    }
    cudaStreamSynchronize(ctx->stream);
    dfree_all(ctx, tmp);
    if (st != BG_OK) return st;
    if (train_step_ms) *train_step_ms = t_train / reps;
    if (infer_ms) *infer_ms = t_infer / reps;
    return BG_OK;
}

bg_status bg_guide_mixture_eval(bg_guide* g, const float* raw, const float* u, const float* w, const float* p_bsdf,
                                size_t n, float* out) {
    if (!g || !g->ctx || (n && (!raw || !u || !w || !p_bsdf || !out))) return BG_ERR_INVALID;
    bg_ctx* ctx = g->ctx;
    if (n == 0) return BG_OK;
    if (n >= (1u << 24)) return fail(ctx, BG_ERR_INVALID, "too many items");
    CK(cudaSetDevice(ctx->device));
    std::vector<void*> tmp;
    void *dr, *du, *dw, *dp, *dout;
    bg_status st = dalloc(ctx, n * bg::GUIDE_HEAD_OUT * sizeof(float), &dr, &tmp);
    if (st == BG_OK) st = dalloc(ctx, n * 3 * sizeof(float), &du, &tmp);
    if (st == BG_OK) st = dalloc(ctx, n * 3 * sizeof(float), &dw, &tmp);
    if (st == BG_OK) st = dalloc(ctx, n * sizeof(float), &dp, &tmp);
    if (st == BG_OK) st = dalloc(ctx, n * 48 * sizeof(float), &dout, &tmp);
    if (st == BG_OK) {
        cudaMemcpyAsync(dr, raw, n * bg::GUIDE_HEAD_OUT * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
        cudaMemcpyAsync(du, u, n * 3 * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
        cudaMemcpyAsync(dw, w, n * 3 * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
        cudaMemcpyAsync(dp, p_bsdf, n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
        bg::launch_guide_mixture_eval((const float*)dr, (const float*)du, (const float*)dw, (const float*)dp,
                                      (uint32_t)n, g->o.alpha, (float*)dout, ctx->stream);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, n * 48 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) st = cuda_fail(ctx, e, "k_guide_mixture_eval");
    }
    cudaStreamSynchronize(ctx->stream);
    dfree_all(ctx, tmp);
    return st;
}

bg_status bg_render_guided(bg_ctx* ctx, const bg_scene* s, bg_guide* g, const bg_camera* cam, const bg_render_opts* o,
                           float* rgb_out, bg_render_stats* stats, bg_guide_stats* gstats) {
    bg_status st = validate_render(ctx, s, cam, o, rgb_out);
    if (st != BG_OK) return st;
    if (!g || g->ctx != ctx) return fail(ctx, BG_ERR_INVALID, "guide does not belong to this context");
    if (o->mode != BG_MODE_PBRT) return fail(ctx, BG_ERR_UNSUPPORTED, "guided rendering needs BG_MODE_PBRT");
    if (s->kind != BG_BVH_WIDE && s->kind != BG_BVH_WIDE2)
        return fail(ctx, BG_ERR_UNSUPPORTED, "guided rendering needs a wide BVH layout");
    if (o->flags & (BG_RENDER_GRAPH | BG_RENDER_STAGE_TIMING))
        return fail(ctx, BG_ERR_UNSUPPORTED, "guided rendering takes no GRAPH or STAGE_TIMING flag");
    if (o->integrator != BG_INTEGRATOR_PATH)
        return fail(ctx, BG_ERR_UNSUPPORTED, "guided rendering runs the path integrator only");
    CK(cudaSetDevice(ctx->device));
    if ((st = ensure_film(ctx, cam->width, cam->height)) != BG_OK) return st;
    if (!(o->flags & BG_RENDER_ACCUMULATE)) {
        bg::launch_clear_film(ctx->film, ctx->stream);
        CK(cudaMemsetAsync(ctx->film.nan_count, 0, sizeof(unsigned long long), ctx->stream));
    }
    const uint64_t npix = (uint64_t)cam->width * cam->height;
    const uint32_t pass_spp = (uint32_t)std::max<uint64_t>(1, g->o.pass_paths / npix);
    const uint32_t cap = (uint32_t)std::min<uint64_t>(ctx->max_queue, npix * std::min(pass_spp, std::max(o->spp, 1u)));
    if ((st = ensure_wave(ctx, cap)) != BG_OK) return st;
    if ((st = ensure_guide_wave(g, cap)) != BG_OK) return st;
    if ((st = ensure_pass(g, npix)) != BG_OK) return st;
    bg::FilmBuffers film = ctx->film;
    film.pass = g->pass;
    const bg::Camera dc = make_camera(*cam);
    bg::GuideWave gw{};
    gw.pool_cap = g->pool_cap;
    gw.cap = g->wcap;  // >= cap, the paths of one wave
    float lo[3], inv[3];
    scene_bounds(s, lo, inv);
    gw.bmin = make_float4(lo[0], lo[1], lo[2], 0.0f);
    gw.binv = make_float4(inv[0], inv[1], inv[2], 0.0f);
    gw.rec = g->rec;
    gw.lrec = g->lrec;
    gw.query = g->query;
    gw.raw = g->raw;
    gw.pool = g->pool;
    gw.ctr = g->ctr;
    gw.wpack = g->wpack;
    const bool train = !(g->o.flags & BG_GUIDE_NO_TRAIN);
    const bool allow_fallback = !(g->o.flags & BG_GUIDE_NO_FALLBACK);
    bg_guide_stats gs{};
    uint64_t launches = 0;
    CK(cudaMemsetAsync(ctx->wave.ray_stats, 0, 4 * sizeof(unsigned long long), ctx->stream));
    CK(cudaEventRecord(g->ev[3], ctx->stream));
    unsigned long long rays[2] = {0, 0};
    uint32_t done = 0;
    for (; done < o->spp && !g->fallback;) {
        const uint32_t k = std::min(pass_spp, o->spp - done);
        const bool guided = g->passes_total >= g->o.warmup_passes && !g->fallback;
        const bool record = train && !g->fallback;
        gw.flags = (record ? bg::GW_RECORD : 0u) | (guided ? bg::GW_GUIDED : 0u) |
                   ((g->o.flags & BG_GUIDE_NO_CONTINUATION) ? 0u : bg::GW_CONT) | ((g->o.flags & BG_GUIDE_NO_NEE) ? 0u : bg::GW_NEE);
        gw.keep_prob = g->keep;
        CK(cudaMemsetAsync(g->ctr, 0, 2 * sizeof(uint32_t), ctx->stream));
        CK(cudaMemsetAsync(g->relvar, 0, 2 * sizeof(double), ctx->stream));
        CK(cudaMemsetAsync(g->pass, 0, npix * 3 * sizeof(float), ctx->stream));
        CK(cudaEventRecord(g->ev[0], ctx->stream));
        bg::RenderParams rp{cam->width, cam->height, k, o->max_depth, o->first_sample + done, o->rr_threshold, o->seed,
                            {lo[0], lo[1], lo[2]}, {inv[0], inv[1], inv[2]}};
        rp = bg::with_camera(rp, dc, o->spp);
        // the stratified sampler's strata follow the global sample index (blocks of x * y samples),
        // so passes of k samples keep them
        bg::strat_params(o->sampler, o->spp, o->x_pixel_samples, o->y_pixel_samples, o->sampled_dimensions,
                         o->jitter_samples, &rp.strat);
        const uint64_t items = npix * k;
        for (uint64_t item0 = 0; item0 < items; item0 += cap) {
            uint32_t nitems = (uint32_t)std::min<uint64_t>(cap, items - item0);
            launches += (uint64_t)bg::launch_wave(s->dev, dc, rp, film, ctx->wave, item0, nitems, ctx->d_err, ctx->shape,
                                                  ctx->stream, nullptr, &gw);
        }
        done += k;
        bg::launch_pass_relvar(film, k, g->relvar, ctx->stream);
        launches += 1;
        CK(cudaGetLastError());
        CK(cudaEventRecord(g->ev[1], ctx->stream));
        uint32_t ctr[2] = {0, 0};
        double rv[2] = {0, 0};
        CK(cudaMemcpyAsync(ctr, g->ctr, sizeof(ctr), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(rv, g->relvar, sizeof(rv), cudaMemcpyDeviceToHost, ctx->stream));
        if ((st = guide_error(ctx)) != BG_OK) return st;  // synchronises the stream
        float pass_ms = 0.0f;
        CK(cudaEventElapsedTime(&pass_ms, g->ev[0], g->ev[1]));
        gs.render_ms += pass_ms;
        gs.passes += 1;
        g->passes_total += 1;
        gs.guided_passes += guided ? 1 : 0;
        gs.records += ctr[0];
        const uint32_t pool_n = std::min(ctr[1], g->pool_cap);
        g->pool_n = pool_n;
        gs.pool_samples += pool_n;
        // ctr[0] counts the positive records of the paths chosen with probability keep: scale the
        // choice so that the next pass fills about pool_cap samples
        g->keep = ctr[0] > 0 ? std::min(1.0f, (float)g->pool_cap * g->keep / (float)ctr[0]) : 1.0f;
        float train_ms = 0.0f;
        if (record && pool_n >= 128) {
            int nb = train_batches(g, g->pool, pool_n, g->o.epochs, &g->epochs_done);
            launches += g->o.epochs + 2 * (uint64_t)nb;
            CK(cudaGetLastError());
            CK(cudaEventRecord(g->ev[2], ctx->stream));
            float ls[2] = {0, 0};
            CK(cudaMemcpyAsync(ls, g->stats, sizeof(ls), cudaMemcpyDeviceToHost, ctx->stream));
            if ((st = guide_error(ctx)) != BG_OK) return st;
            CK(cudaEventElapsedTime(&train_ms, g->ev[1], g->ev[2]));
            gs.train_ms += train_ms;
            gs.adam_steps += (uint32_t)nb;
            gs.last_loss = ls[0] / (double)nb;  // mean batch loss of this pass's steps
        }
        // variance bookkeeping (relative variance per sample of this pass, see k_pass_relvar)
        if (rv[1] > 0.0) {
            const double relvar = rv[0] / rv[1];
            if (guided) {
                g->rv_guided[g->n_guided % bg_guide::kWindow] = relvar;
                g->ms_guided[g->n_guided % bg_guide::kWindow] = pass_ms + train_ms;
                g->n_guided += 1;
            } else if (!g->fallback) {
                g->rv_plain_sum += relvar;
                g->ms_plain_sum += pass_ms;
                g->n_plain += 1;
            }
        }
        if (guided && allow_fallback && g->n_plain >= 1 && g->n_guided >= 2 * bg_guide::kWindow) {
            const uint32_t k = std::min(g->n_guided, bg_guide::kWindow);
            double a = 0, b = 0;
            for (uint32_t i = 0; i < k; ++i) {
                a += g->rv_guided[i];
                b += g->ms_guided[i];
            }
            if ((a / k) * (b / k) >= (g->rv_plain_sum / g->n_plain) * (g->ms_plain_sum / g->n_plain)) g->fallback = true;
        }
    }
    if (g->n_plain) {
        gs.relvar_plain = g->rv_plain_sum / g->n_plain;
        gs.ms_plain = g->ms_plain_sum / g->n_plain;
    }
    if (g->n_guided) {
        const uint32_t k = std::min(g->n_guided, bg_guide::kWindow);
        for (uint32_t i = 0; i < k; ++i) {
            gs.relvar_guided += g->rv_guided[i] / k;
            gs.ms_guided += g->ms_guided[i] / k;
        }
    }
    gs.fallback = g->fallback ? 1u : 0u;
    if (done < o->spp) {
        // after the fallback: the rest of the samples through the plain graph-captured wavefront
        bg_render_opts po = *o;
        po.spp = o->spp - done;
        po.first_sample = o->first_sample + done;
        po.flags = BG_RENDER_ACCUMULATE | BG_RENDER_NO_READBACK | BG_RENDER_GRAPH;
        bg_render_stats ps{};
        CK(cudaMemcpyAsync(rays, ctx->wave.ray_stats, sizeof(rays), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        if ((st = bg_render(ctx, s, cam, &po, nullptr, &ps)) != BG_OK) return st;
        gs.render_ms += ps.device_ms;
        launches += ps.launches;
        rays[0] += ps.extension_rays;
        rays[1] += ps.shadow_rays;
    } else {
        CK(cudaMemcpyAsync(rays, ctx->wave.ray_stats, sizeof(rays), cudaMemcpyDeviceToHost, ctx->stream));
    }
    bg::launch_resolve(ctx->film, ctx->stream);
    launches += 1;
    CK(cudaGetLastError());
    CK(cudaEventRecord(g->ev[4], ctx->stream));
    uint32_t word = 0;
    st = check_device_error(ctx, &word);
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, g->ev[3], g->ev[4]);
        stats->device_ms = ms;
        stats->samples = npix * o->spp;
        stats->launches = launches;
        stats->error_word = word;
        unsigned long long nan = 0;
        cudaMemcpy(&nan, ctx->film.nan_count, sizeof(nan), cudaMemcpyDeviceToHost);
        stats->nan_samples = nan;
        stats->extension_rays = rays[0];
        stats->shadow_rays = rays[1];
    }
    if (gstats) *gstats = gs;
    if (st != BG_OK) return st;
    if (!(o->flags & BG_RENDER_NO_READBACK)) {
        CK(cudaMemcpyAsync(rgb_out, ctx->film.rgb, npix * 3 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return BG_OK;
}

}  // extern "C"

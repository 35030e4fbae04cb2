// bg_api.cpp - the C ABI of libbonsai_gpu.so (include/bonsai_gpu.h).
//
// Owns the CUDA context state (stream, events, device buffers with an optional memory cap),
// the scene builder (host copies -> BVH build -> device upload) and the render driver that
// replaces SamplerIntegrator::render (src/base/integrator.rs:35-133).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/bonsai_gpu.h"
#include "bg_bvh.h"
#include "bg_internal.h"
#include "bg_kernels.h"

namespace bgi {

bg_status fail(bg_ctx* c, bg_status s, const std::string& msg) {
    if (c) c->err = msg;
    return s;
}
bg_status cuda_fail(bg_ctx* c, cudaError_t e, const char* what) {
    return fail(c, e == cudaErrorMemoryAllocation ? BG_ERR_OOM : BG_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}
bg_status dalloc(bg_ctx* ctx, size_t bytes, void** p, std::vector<void*>* owner) {
    if (ctx->cap && ctx->used + bytes > ctx->cap)
        return fail(ctx, BG_ERR_OOM, "device memory cap exceeded (" + std::to_string(ctx->used + bytes) + " > " +
                                         std::to_string(ctx->cap) + " bytes)");
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc");
    ctx->used += bytes;
    ctx->sizes[*p] = bytes;
    if (owner) owner->push_back(*p);
    return BG_OK;
}
void dfree(bg_ctx* ctx, void* p) {
    auto it = ctx->sizes.find(p);
    if (it != ctx->sizes.end()) {
        ctx->used -= it->second;
        ctx->sizes.erase(it);
    }
    cudaFree(p);
}
void dfree_all(bg_ctx* ctx, std::vector<void*>& v) {
    for (void* p : v) dfree(ctx, p);
    v.clear();
}
template <class T>
bg_status upload(bg_ctx* ctx, const std::vector<T>& h, const T** d, std::vector<void*>* owner) {
    void* p = nullptr;
    bg_status s = dalloc(ctx, h.size() * sizeof(T), &p, owner);
    if (s != BG_OK) return s;
    if (!h.empty()) {
        cudaError_t e = cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemcpyAsync");
    }
    *d = static_cast<const T*>(p);
    return BG_OK;
}

// ---- camera transforms (src/base/transform.rs, src/cameras/perspective.rs:49-113), f32
struct M4 {
    float m[4][4];
};
M4 ident() {
    M4 r{};
    for (int i = 0; i < 4; ++i) r.m[i][i] = 1.0f;
    return r;
}
M4 mul(const M4& a, const M4& b) {
    M4 r{};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j] + a.m[i][3] * b.m[3][j];
    return r;
}
M4 inverse(const M4& in) {  // Gauss-Jordan with full pivoting (mat4.rs:72-140)
    float a[4][4];
    std::memcpy(a, in.m, sizeof(a));
    int ic[4] = {0}, ir[4] = {0}, piv[4] = {0};
    for (int i = 0; i < 4; ++i) {
        int row = 0, col = 0;
        float big = 0.0f;
        for (int j = 0; j < 4; ++j)
            if (piv[j] != 1)
                for (int k = 0; k < 4; ++k)
                    if (piv[k] == 0 && std::fabs(a[j][k]) >= big) {
                        big = std::fabs(a[j][k]);
                        row = j;
                        col = k;
                    }
        piv[col] += 1;
        if (row != col)
            for (int k = 0; k < 4; ++k) std::swap(a[row][k], a[col][k]);
        ir[i] = row;
        ic[i] = col;
        float pinv = 1.0f / a[col][col];
        a[col][col] = 1.0f;
        for (int j = 0; j < 4; ++j) a[col][j] *= pinv;
        for (int j = 0; j < 4; ++j)
            if (j != col) {
                float save = a[j][col];
                a[j][col] = 0.0f;
                for (int k = 0; k < 4; ++k) a[j][k] -= a[col][k] * save;
            }
    }
    for (int j = 3; j >= 0; --j)
        if (ir[j] != ic[j])
            for (int k = 0; k < 4; ++k) std::swap(a[k][ir[j]], a[k][ic[j]]);
    M4 r;
    std::memcpy(r.m, a, sizeof(a));
    return r;
}
struct Xf {
    M4 m, mi;
};
Xf xmul(const Xf& a, const Xf& b) { return {mul(a.m, b.m), mul(b.mi, a.mi)}; }
Xf xinv(const Xf& a) { return {a.mi, a.m}; }
Xf xscale(float x, float y, float z) {
    Xf t{ident(), ident()};
    t.m.m[0][0] = x;
    t.m.m[1][1] = y;
    t.m.m[2][2] = z;
    t.mi.m[0][0] = 1.0f / x;
    t.mi.m[1][1] = 1.0f / y;
    t.mi.m[2][2] = 1.0f / z;
    return t;
}
Xf xtranslate(float x, float y, float z) {
    Xf t{ident(), ident()};
    t.m.m[0][3] = x;
    t.m.m[1][3] = y;
    t.m.m[2][3] = z;
    t.mi.m[0][3] = -x;
    t.mi.m[1][3] = -y;
    t.mi.m[2][3] = -z;
    return t;
}
struct F3 {
    float x, y, z;
};
F3 sub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
float len(F3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
F3 nrm(F3 a) {
    float inv = 1.0f / len(a);
    return {a.x * inv, a.y * inv, a.z * inv};
}
F3 crs(F3 a, F3 b) {  // vec3.rs:108-122 (f64 products, rounded once)
    double x = a.x, y = a.y, z = a.z, vx = b.x, vy = b.y, vz = b.z;
    return {(float)(y * vz - z * vy), (float)(z * vx - x * vz), (float)(x * vy - y * vx)};
}
F3 xf_point_h(const float (&m)[4][4], float x, float y, float z) {  // Point3::transform (point3.rs:51-69)
    float xp = m[0][0] * x + m[0][1] * y + m[0][2] * z + m[0][3];
    float yp = m[1][0] * x + m[1][1] * y + m[1][2] * z + m[1][3];
    float zp = m[2][0] * x + m[2][1] * y + m[2][2] * z + m[2][3];
    float wp = m[3][0] * x + m[3][1] * y + m[3][2] * z + m[3][3];
    if (wp == 1.0f) return {xp, yp, zp};
    float inv = 1.0f / wp;
    return {xp * inv, yp * inv, zp * inv};
}
bg::Camera make_camera(const bg_camera& c) {
    bg::Camera out{};
    float rx = (float)c.width, ry = (float)c.height;
    // Transform::perspective (transform.rs:48-73)
    M4 p = ident();
    float f = c.far_plane, n = c.near_plane;
    p.m[2][2] = f / (f - n);
    p.m[2][3] = -f * n / (f - n);
    p.m[3][2] = 1.0f;
    p.m[3][3] = 0.0f;
    float inv_tan = 1.0f / std::tan(c.fov_deg * (3.14159265358979323846f / 180.0f) / 2.0f);
    Xf c2s = xmul(xscale(inv_tan, inv_tan, 1.0f), Xf{p, inverse(p)});
    float sx0, sx1, sy0, sy1, frame = rx / ry;
    if (frame > 1.0f) {
        sx0 = -frame; sx1 = frame; sy0 = -1.0f; sy1 = 1.0f;
    } else {
        sx0 = -1.0f; sx1 = 1.0f; sy0 = -1.0f / frame; sy1 = 1.0f / frame;
    }
    Xf s2r = xmul(xmul(xscale(rx, ry, 1.0f), xscale(1.0f / (sx1 - sx0), 1.0f / (sy0 - sy1), 1.0f)),
                  xtranslate(-sx0, -sy1, 0.0f));
    Xf r2c = xmul(xinv(c2s), xinv(s2r));
    std::memcpy(out.r2c, r2c.m.m, sizeof(out.r2c));
    // Transform::look_at (transform.rs:152-189) = camera_to_world
    M4 cw = ident();
    F3 pos{c.position[0], c.position[1], c.position[2]}, look{c.look_at[0], c.look_at[1], c.look_at[2]};
    F3 up{c.up[0], c.up[1], c.up[2]};
    cw.m[0][3] = pos.x;
    cw.m[1][3] = pos.y;
    cw.m[2][3] = pos.z;
    cw.m[3][3] = 1.0f;
    F3 dir = nrm(sub(look, pos));
    if (len(crs(nrm(up), dir)) != 0.0f) {
        F3 right = nrm(crs(nrm(up), dir));
        F3 nup = crs(dir, right);
        cw.m[0][0] = right.x; cw.m[1][0] = right.y; cw.m[2][0] = right.z; cw.m[3][0] = 0.0f;
        cw.m[0][1] = nup.x; cw.m[1][1] = nup.y; cw.m[2][1] = nup.z; cw.m[3][1] = 0.0f;
        cw.m[0][2] = dir.x; cw.m[1][2] = dir.y; cw.m[2][2] = dir.z; cw.m[3][2] = 0.0f;
    } else {
        cw = ident();
    }
    std::memcpy(out.c2w, cw.m, sizeof(out.c2w));
    out.width = c.width;
    out.height = c.height;
    // dx_camera / dy_camera (perspective.rs:86-89): Point3::transform of (1,0,0) / (0,1,0) minus
    // that of the origin
    const F3 o = xf_point_h(r2c.m.m, 0.0f, 0.0f, 0.0f), px = xf_point_h(r2c.m.m, 1.0f, 0.0f, 0.0f),
             py = xf_point_h(r2c.m.m, 0.0f, 1.0f, 0.0f);
    const F3 dx = sub(px, o), dy = sub(py, o);
    out.dxc[0] = dx.x; out.dxc[1] = dx.y; out.dxc[2] = dx.z;
    out.dyc[0] = dy.x; out.dyc[1] = dy.y; out.dyc[2] = dy.z;
    out.lens_radius = c.lens_radius;
    out.focal_distance = c.focal_distance;
    return out;
}

// TrowbridgeReitzDistribution::roughness_to_alpha (src/base/microfacet.rs:45-53)
float roughness_to_alpha(float r) {
    r = std::fmax(r, 1e-3f);
    float x = std::log(r);
    return 1.62142f + 0.819955f * x + 0.1734f * x * x + 0.0171201f * x * x * x + 0.000640711f * x * x * x * x;
}

bg_status ensure_film(bg_ctx* ctx, uint32_t w, uint32_t h) {
    if (ctx->film_w == w && ctx->film_h == h && ctx->film.sum) return BG_OK;
    dfree_all(ctx, ctx->film_allocs);
    ctx->film = bg::FilmBuffers{};
    ctx->film_w = ctx->film_h = 0;
    size_t npix = (size_t)w * h;
    void *a, *b, *c, *d, *e;
    bg_status s;
    if ((s = dalloc(ctx, npix * 3 * sizeof(double), &a, &ctx->film_allocs)) != BG_OK) return s;
    if ((s = dalloc(ctx, npix * 3 * sizeof(double), &b, &ctx->film_allocs)) != BG_OK) return s;
    if ((s = dalloc(ctx, npix * sizeof(uint32_t), &c, &ctx->film_allocs)) != BG_OK) return s;
    if ((s = dalloc(ctx, npix * 3 * sizeof(float), &d, &ctx->film_allocs)) != BG_OK) return s;
    if ((s = dalloc(ctx, sizeof(unsigned long long), &e, &ctx->film_allocs)) != BG_OK) return s;
    ctx->film.sum = (double*)a;
    ctx->film.sumsq = (double*)b;
    ctx->film.count = (uint32_t*)c;
    ctx->film.rgb = (float*)d;
    ctx->film.nan_count = (unsigned long long*)e;
    ctx->film.npix = (uint32_t)npix;
    ctx->film_w = w;
    ctx->film_h = h;
    bg::launch_clear_film(ctx->film, ctx->stream);
    CK(cudaMemsetAsync(e, 0, sizeof(unsigned long long), ctx->stream));
    return BG_OK;
}

bg_status ensure_wave(bg_ctx* ctx, uint32_t cap) {
    const bool half = ctx->shape.shadow_half != 0;
    if (ctx->wave.capacity >= cap && ctx->wave.ray_o && (ctx->wave.sh_capacity == ctx->wave.capacity) == half)
        return BG_OK;
    dfree_all(ctx, ctx->wave_allocs);
    ctx->wave = bg::WaveBuffers{};
    bg::WaveBuffers& w = ctx->wave;
    auto get = [&](size_t bytes, void** p) { return dalloc(ctx, bytes, p, &ctx->wave_allocs); };
    bg_status s;
    size_t n = cap;
#define WB(field, bytes)                                   \
    do {                                                   \
        void* p_;                                          \
        if ((s = get((bytes), &p_)) != BG_OK) return s;    \
        w.field = (decltype(w.field))p_;                   \
    } while (0)
    WB(ray_o, n * sizeof(float4));
    WB(ray_d, n * sizeof(float4));
    WB(hit, n * sizeof(int2));
    WB(pixel, n * sizeof(uint32_t));
    WB(sample, n * sizeof(uint32_t));
    WB(state, n * sizeof(uint32_t));
    WB(beta, n * sizeof(float4));
    WB(L, n * sizeof(float4));
    WB(nee_beta, n * sizeof(float4));
    WB(pending, 2 * n * sizeof(float4));
    const size_t nsh = half ? n : 2 * n;
    WB(sh_o, nsh * sizeof(float4));
    WB(sh_d, nsh * sizeof(float4));
    WB(sh_ref, nsh * sizeof(uint32_t));
    WB(queue[0], n * sizeof(uint32_t));
    WB(queue[1], n * sizeof(uint32_t));
    WB(cls_queue, 5 * n * sizeof(uint32_t));
    WB(done, n * sizeof(uint32_t));
    WB(counters, 16 * sizeof(uint32_t));
    WB(ray_stats, 4 * sizeof(unsigned long long));
    WB(wavectl, 4 * sizeof(uint32_t));
    WB(scene_id, n * sizeof(uint32_t));
    WB(qsort, n * sizeof(uint32_t));
    WB(sort_hist, 8192 * sizeof(uint32_t));
#undef WB
    w.capacity = cap;
    w.sh_capacity = (uint32_t)nsh;
    if (cudaMemsetAsync(w.sort_hist, 0, 8192 * sizeof(uint32_t), ctx->stream) != cudaSuccess)
        return fail(ctx, BG_ERR_CUDA, "cudaMemsetAsync");
    return BG_OK;
}

// L2 access-policy window over the scene's 8-wide traversal range (nodes + leaf primitives): its
// lines persist in the L2 set-aside while the wave state streams past them.  The set-aside is
// requested for the render and given back after it (limit 0, persisting lines reset), so nothing
// outlasts the call.
void l2_window(bg_ctx* ctx, const bg_scene* s, bool on) {
    if (!ctx->shape.l2_persist) return;
    if (ctx->l2_window_max == 0 && ctx->l2_persist_max == 0) {
        int persist = 0, window = 0;
        cudaDeviceGetAttribute(&persist, cudaDevAttrMaxPersistingL2CacheSize, ctx->device);
        cudaDeviceGetAttribute(&window, cudaDevAttrMaxAccessPolicyWindowSize, ctx->device);
        ctx->l2_persist_max = (size_t)std::max(persist, 0);
        ctx->l2_window_max = (size_t)std::max(window, 0);
    }
    cudaStreamAttrValue a;
    std::memset(&a, 0, sizeof(a));
    const bool use = on && s && s->hot && ctx->l2_persist_max && ctx->l2_window_max;
    if (use) {
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, ctx->l2_persist_max);
        const size_t n = std::min(s->hot_bytes, ctx->l2_window_max);
        a.accessPolicyWindow.base_ptr = s->hot;
        a.accessPolicyWindow.num_bytes = n;
        a.accessPolicyWindow.hitRatio = (float)std::min(1.0, (double)ctx->l2_persist_max / (double)n);
        a.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
        a.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    }
    cudaStreamSetAttribute(ctx->stream, cudaStreamAttributeAccessPolicyWindow, &a);
    if (!use) {
        cudaStreamSynchronize(ctx->stream);
        cudaCtxResetPersistingL2Cache();
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0);
    }
}

// Tree wavefront buffers for `samples` camera samples per wave: two level queues of 2 x samples
// nodes each (node differentials only for textured scenes), `sh_cap` shadow rays, one
// accumulator per sample.
bg_status ensure_tree_wave(bg_ctx* ctx, uint32_t samples, uint32_t sh_cap, bool textured) {
    bg::TreeWave& t = ctx->tree;
    const uint32_t cap = 2 * samples;
    if (t.counters && t.samp_cap >= samples && t.cap >= cap && t.sh_cap >= sh_cap && (t.textured || !textured))
        return BG_OK;
    dfree_all(ctx, ctx->tree_allocs);
    t = bg::TreeWave{};
    auto get = [&](size_t bytes, void** p) { return dalloc(ctx, bytes, p, &ctx->tree_allocs); };
    bg_status s;
#define TW(field, bytes)                                   \
    do {                                                   \
        void* p_;                                          \
        if ((s = get((bytes), &p_)) != BG_OK) return s;    \
        t.field = (decltype(t.field))p_;                   \
    } while (0)
    for (int b = 0; b < 2; ++b) {
        TW(ray_o[b], (size_t)cap * sizeof(float4));
        TW(ray_d[b], (size_t)cap * sizeof(float4));
        TW(beta[b], (size_t)cap * sizeof(float4));
        TW(meta[b], (size_t)cap * sizeof(uint4));
        if (textured) TW(rd[b], 4 * (size_t)cap * sizeof(float4));
    }
    TW(hit, (size_t)cap * sizeof(int2));
    TW(sh_o, (size_t)sh_cap * sizeof(float4));
    TW(sh_d, (size_t)sh_cap * sizeof(float4));
    TW(sh_c, (size_t)sh_cap * sizeof(float4));
    TW(L, (size_t)samples * sizeof(float4));
    TW(counters, 8 * sizeof(uint32_t));
    TW(ray_stats, 2 * sizeof(unsigned long long));
#undef TW
    t.cap = cap;
    t.sh_cap = sh_cap;
    t.samp_cap = samples;
    t.textured = textured ? 1u : 0u;
    return BG_OK;
}

bg_status check_device_error(bg_ctx* ctx, uint32_t* word) {
    uint32_t e = 0;
    CK(cudaMemcpyAsync(&e, ctx->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (word) *word = e;
    if (e) {
        CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(uint32_t), ctx->stream));
        static const char* names[] = {"traversal stack overflow", "queue overflow", "bad primitive index",
                                      "bad node index", "guide wait timed out"};
        std::string what;
        for (int b = 0; b < 5; ++b)
            if (e & (1u << b)) what += (what.empty() ? "" : ", ") + std::string(names[b]);
        return fail(ctx, BG_ERR_DEVICE, "device error word " + std::to_string(e) + ": " + what);
    }
    return BG_OK;
}

// Inverse of an affine 3x4 transform through the 4x4 Gauss-Jordan inverse (mat4.rs:72-140), as
// Transform::new(m) computes m_inverse.
extern "C++" void affine_inverse(const float* xf, float* inv) {
    M4 m = ident();
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) m.m[r][c] = xf[4 * r + c];
    M4 mi = inverse(m);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) inv[4 * r + c] = mi.m[r][c];
}

// Per-triangle bits for next-event estimation (TRI_LFLIP, TRI_SFLIP): whether the surface normal
// of a hit (triangle.rs:299-307, then face-forwarded to the shading normal by
// set_shading_geometry) and of a sampled point (triangle.rs:534-545) point against
// cross(p1 - p0, p2 - p0).  With vertex normals both follow the sign of dot(ng, sum b_i n_i),
// fixed over the triangle when the three dot(ng, n_i) share a sign; an emitting triangle whose
// vertex normals straddle its plane is refused (its emission side would change across it).
extern "C++" bool triangle_light_sides(const bg_scene* s, std::vector<uint8_t>* out, std::string* why) {
    const size_t ntri = s->tri_mat.size();
    out->resize(ntri);
    for (size_t i = 0; i < ntri; ++i) {
        uint8_t f = s->tri_flags[i];
        const bool flip = ((f & bg::TRI_REVERSE) != 0) != ((f & bg::TRI_SWAPS) != 0);
        if (!(f & bg::TRI_NORMALS)) {
            if (flip) f |= bg::TRI_LFLIP | bg::TRI_SFLIP;
            (*out)[i] = f;
            continue;
        }
        const float* p = &s->tri[9 * i];
        const double e1[3] = {(double)p[3] - p[0], (double)p[4] - p[1], (double)p[5] - p[2]};
        const double e2[3] = {(double)p[6] - p[0], (double)p[7] - p[1], (double)p[8] - p[2]};
        const double ng[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        int pos = 0, neg = 0;
        for (int k = 0; k < 3; ++k) {
            const float* n = &s->tri_n[9 * i + 3 * k];
            const double d = ng[0] * n[0] + ng[1] * n[1] + ng[2] * n[2];
            pos += d > 0.0;
            neg += d < 0.0;
        }
        if (pos == 3 || neg == 3) {
            const bool against = neg == 3;
            // hit: the shading normal is the interpolated one, negated for reverse_orientation
            if (against != ((f & bg::TRI_REVERSE) != 0)) f |= bg::TRI_LFLIP;
            if (against) f |= bg::TRI_SFLIP;
        } else if (s->tri_light[i] >= 0) {
            *why = "emitting triangle " + std::to_string(i) +
                   " has vertex normals on both sides of its plane (its emission side would vary across it)";
            return false;
        }
        (*out)[i] = f;
    }
    return true;
}

}  // namespace bgi

using namespace bgi;

namespace bg {
// Scene internals for the allocation-free render entry point (bg_noalloc.cu).
bool scene_device_view(const bg_scene* s, Scene* dev, uint32_t* kind, int* device) {
    if (!s || !s->ctx || !s->committed) return false;
    *dev = s->dev;
    *kind = s->kind;
    *device = s->ctx->device;
    return true;
}
void scene_set_error(const bg_scene* s, const std::string& msg) {
    if (s && s->ctx) s->ctx->err = msg;
}
Camera camera_for(const bg_camera& c) { return make_camera(c); }
}  // namespace bg

extern "C" {

const char* bg_status_string(bg_status s) {
    switch (s) {
        case BG_OK: return "ok";
        case BG_ERR_INVALID: return "invalid argument";
        case BG_ERR_CUDA: return "CUDA error";
        case BG_ERR_OOM: return "out of device memory";
        case BG_ERR_TIMEOUT: return "device wait timed out";
        case BG_ERR_DEVICE: return "device-side error";
        case BG_ERR_UNSUPPORTED: return "unsupported";
        case BG_ERR_NO_DEVICE: return "no usable CUDA device";
    }
    return "unknown status";
}

const char* bg_last_error(const bg_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

bg_status bg_create(const bg_device_opts* opts, bg_ctx** out) {
    if (!out) return BG_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return BG_ERR_NO_DEVICE;
    }
    bg_ctx* ctx = new bg_ctx();
    ctx->device = opts ? opts->device : 0;
    if (ctx->device < 0 || ctx->device >= ndev) {
        delete ctx;
        return BG_ERR_INVALID;
    }
    if (opts) {
        ctx->cap = opts->memory_cap_bytes;
        if (opts->max_queue_paths) ctx->max_queue = opts->max_queue_paths;
        if (opts->block_size) ctx->shape.block = (int)opts->block_size;
    }
    auto bail = [&](cudaError_t e) {
        bg_status s = (e == cudaErrorNoKernelImageForDevice || e == cudaErrorInvalidDevice) ? BG_ERR_NO_DEVICE
                                                                                             : BG_ERR_CUDA;
        bg_destroy(ctx);
        return s;
    };
    cudaError_t e;
    if ((e = cudaSetDevice(ctx->device)) != cudaSuccess) return bail(e);
    cudaDeviceProp prop;
    if ((e = cudaGetDeviceProperties(&prop, ctx->device)) != cudaSuccess) return bail(e);
    ctx->shape.sms = prop.multiProcessorCount;
    if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e);
    for (auto& st : ctx->fork.aux)
        if ((e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess) return bail(e);
    if ((e = cudaEventCreateWithFlags(&ctx->fork.fork, cudaEventDisableTiming)) != cudaSuccess) return bail(e);
    for (auto& ev : ctx->fork.join)
        if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) return bail(e);
    ctx->shape.fork = &ctx->fork;  // BG_TUNE_CONCURRENT_SHADE, on by default
    if ((e = cudaEventCreate(&ctx->ev_begin)) != cudaSuccess) return bail(e);
    if ((e = cudaEventCreate(&ctx->ev_end)) != cudaSuccess) return bail(e);
    for (auto& ev : ctx->stage_ev)
        if ((e = cudaEventCreate(&ev)) != cudaSuccess) return bail(e);
    void* p;
    if (dalloc(ctx, 64, &p, &ctx->user) != BG_OK) return bail(cudaErrorMemoryAllocation);
    ctx->d_err = (uint32_t*)p;
    ctx->d_counters = (unsigned long long*)((char*)p + 16);
    ctx->d_head = (uint32_t*)((char*)p + 32);
    if ((e = cudaMemsetAsync(p, 0, 64, ctx->stream)) != cudaSuccess) return bail(e);
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return bail(e);
    *out = ctx;
    return BG_OK;
}

void bg_destroy(bg_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (bg_scene* s : ctx->scenes) {  // scenes outliving their context keep only host state
        dfree_all(ctx, s->allocs);
        s->ctx = nullptr;
        s->committed = false;
    }
    ctx->scenes.clear();
    guide_orphan_all(ctx);
    dfree_all(ctx, ctx->wave_allocs);
    dfree_all(ctx, ctx->tree_allocs);
    dfree_all(ctx, ctx->film_allocs);
    dfree_all(ctx, ctx->user);
    if (ctx->flush) cudaFree(ctx->flush);
    if (ctx->ev_begin) cudaEventDestroy(ctx->ev_begin);
    if (ctx->ev_end) cudaEventDestroy(ctx->ev_end);
    for (auto ev : ctx->stage_ev)
        if (ev) cudaEventDestroy(ev);
    for (auto ev : ctx->timing_ev) cudaEventDestroy(ev);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->batch_graph) cudaGraphExecDestroy(ctx->batch_graph);
    dfree_all(ctx, ctx->batch_allocs);
    for (auto st : ctx->fork.aux)
        if (st) cudaStreamDestroy(st);
    if (ctx->fork.fork) cudaEventDestroy(ctx->fork.fork);
    for (auto ev : ctx->fork.join)
        if (ev) cudaEventDestroy(ev);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

bg_status bg_synchronize(bg_ctx* ctx) {
    if (!ctx) return BG_ERR_INVALID;
    CK(cudaStreamSynchronize(ctx->stream));
    return BG_OK;
}

bg_status bg_flush_l2(bg_ctx* ctx) {
    if (!ctx) return BG_ERR_INVALID;
    if (!ctx->flush) {
        ctx->flush_bytes = (size_t)512 << 20;  // > 4x the 129 MB L2
        CK(cudaMalloc(&ctx->flush, ctx->flush_bytes));
    }
    static unsigned char v = 0;
    CK(cudaMemsetAsync(ctx->flush, ++v, ctx->flush_bytes, ctx->stream));
    return BG_OK;
}

bg_status bg_device_alloc(bg_ctx* ctx, size_t bytes, void** p) {
    if (!ctx || !p) return BG_ERR_INVALID;
    return dalloc(ctx, bytes, p, &ctx->user);
}
bg_status bg_device_free(bg_ctx* ctx, void* p) {
    if (!ctx) return BG_ERR_INVALID;
    auto it = std::find(ctx->user.begin(), ctx->user.end(), p);
    if (it == ctx->user.end()) return fail(ctx, BG_ERR_INVALID, "pointer was not allocated by bg_device_alloc");
    CK(cudaStreamSynchronize(ctx->stream));
    dfree(ctx, p);
    ctx->user.erase(it);
    return BG_OK;
}
bg_status bg_memcpy_h2d(bg_ctx* ctx, void* d, const void* h, size_t bytes) {
    if (!ctx) return BG_ERR_INVALID;
    CK(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return BG_OK;
}
bg_status bg_memcpy_d2h(bg_ctx* ctx, void* h, const void* d, size_t bytes) {
    if (!ctx) return BG_ERR_INVALID;
    CK(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return BG_OK;
}

bg_status bg_get_tuning(const bg_ctx* ctx, bg_tuning* out) {
    if (!ctx || !out) return BG_ERR_INVALID;
    out->wave_paths = ctx->max_queue;
    out->blocks_per_sm = (uint32_t)ctx->shape.blocks_per_sm;
    out->refill = (uint32_t)ctx->shape.refill;
    out->flags = (ctx->shape.sort_rays ? BG_TUNE_SORT_RAYS : 0u) | (ctx->shape.l2_persist ? BG_TUNE_L2_PERSIST : 0u) |
                 (ctx->shape.tile_pixels ? BG_TUNE_TILE_PIXELS : 0u) |
                 (ctx->shape.shadow_half ? BG_TUNE_SHADOW_QUEUE_HALF : 0u) |
                 (ctx->shape.fork ? BG_TUNE_CONCURRENT_SHADE : 0u);
    return BG_OK;
}

bg_status bg_set_tuning(bg_ctx* ctx, const bg_tuning* t) {
    if (!ctx || !t) return BG_ERR_INVALID;
    if (t->wave_paths < 1024 || t->wave_paths > (1u << 26)) return fail(ctx, BG_ERR_INVALID, "wave_paths out of range");
    if (t->blocks_per_sm < 1 || t->blocks_per_sm > 64) return fail(ctx, BG_ERR_INVALID, "blocks_per_sm out of range");
    if (t->refill < 1 || t->refill > 32) return fail(ctx, BG_ERR_INVALID, "refill must be in 1..32");
    ctx->max_queue = t->wave_paths;
    ctx->shape.blocks_per_sm = (int)t->blocks_per_sm;
    ctx->shape.refill = (int)t->refill;
    ctx->shape.sort_rays = (t->flags & BG_TUNE_SORT_RAYS) ? 1 : 0;
    ctx->shape.l2_persist = (t->flags & BG_TUNE_L2_PERSIST) ? 1 : 0;
    ctx->shape.tile_pixels = (t->flags & BG_TUNE_TILE_PIXELS) ? 1 : 0;
    ctx->shape.shadow_half = (t->flags & BG_TUNE_SHADOW_QUEUE_HALF) ? 1 : 0;
    ctx->shape.fork = (t->flags & BG_TUNE_CONCURRENT_SHADE) ? &ctx->fork : nullptr;
    return BG_OK;
}

// ---------------------------------------------------------------- scene
bg_status bg_scene_create(bg_ctx* ctx, bg_scene** out) {
    if (!ctx || !out) return BG_ERR_INVALID;
    *out = new bg_scene();
    (*out)->ctx = ctx;
    ctx->scenes.insert(*out);
    return BG_OK;
}

void bg_scene_destroy(bg_scene* s) {
    if (!s) return;
    if (s->ctx) {
        bg_ctx* ctx = s->ctx;
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        dfree_all(ctx, s->allocs);
        ctx->scenes.erase(s);
    }
    delete s;
}

bg_status bg_scene_add_material(bg_scene* s, const bg_material* m, uint32_t* id) {
    if (!s || !m) return BG_ERR_INVALID;
    if (!s->ctx) return BG_ERR_INVALID;
    if (s->committed) return fail(s->ctx, BG_ERR_INVALID, "scene already committed");
    if (m->type > BG_MAT_DIELECTRIC) return fail(s->ctx, BG_ERR_INVALID, "unknown material type");
    if (m->type == BG_MAT_DIELECTRIC && !(m->ior > 0.0f))
        return fail(s->ctx, BG_ERR_INVALID, "dielectric ior must be > 0");
    if (!std::isfinite(m->sigma)) return fail(s->ctx, BG_ERR_INVALID, "matte sigma must be finite");
    s->mats.push_back(*m);
    if (id) *id = (uint32_t)(s->mats.size() - 1);
    return BG_OK;
}

bg_status bg_scene_add_area_light(bg_scene* s, const bg_area_light* l, uint32_t* id) {
    if (!s || !l) return BG_ERR_INVALID;
    if (!s->ctx) return BG_ERR_INVALID;
    if (s->committed) return fail(s->ctx, BG_ERR_INVALID, "scene already committed");
    s->lights.push_back(*l);
    if (id) *id = (uint32_t)(s->lights.size() - 1);
    return BG_OK;
}

bg_status bg_scene_add_triangle_mesh(bg_scene* s, const float* xyz, size_t ntri, const uint32_t* mat,
                                     const int32_t* light, const float* normals, const float* uvs, uint32_t flags) {
    if (!s || (ntri && (!xyz || !mat))) return BG_ERR_INVALID;
    if (!s->ctx) return BG_ERR_INVALID;
    if (s->committed) return fail(s->ctx, BG_ERR_INVALID, "scene already committed");
    if (flags & ~(BG_TRI_REVERSE_ORIENTATION | BG_TRI_SWAPS_HANDEDNESS))
        return fail(s->ctx, BG_ERR_INVALID, "unknown triangle flags");
    if (s->tri_mat.size() + ntri >= (1ull << 31)) return fail(s->ctx, BG_ERR_INVALID, "too many triangles");
    for (size_t i = 0; i < ntri; ++i) {
        if (mat[i] >= s->mats.size())
            return fail(s->ctx, BG_ERR_INVALID, "triangle " + std::to_string(i) + " has an unknown material id");
        if (light && light[i] >= 0 && (size_t)light[i] >= s->lights.size())
            return fail(s->ctx, BG_ERR_INVALID, "triangle " + std::to_string(i) + " has an unknown light id");
        for (int k = 0; k < 9; ++k)
            if (!std::isfinite(xyz[9 * i + k]))
                return fail(s->ctx, BG_ERR_INVALID, "triangle " + std::to_string(i) + " has a non-finite vertex");
        for (int k = 0; normals && k < 9; ++k)
            if (!std::isfinite(normals[9 * i + k]))
                return fail(s->ctx, BG_ERR_INVALID, "triangle " + std::to_string(i) + " has a non-finite normal");
        for (int k = 0; uvs && k < 6; ++k)
            if (!std::isfinite(uvs[6 * i + k]))
                return fail(s->ctx, BG_ERR_INVALID, "triangle " + std::to_string(i) + " has a non-finite uv");
    }
    s->tri.insert(s->tri.end(), xyz, xyz + 9 * ntri);
    s->tri_mat.insert(s->tri_mat.end(), mat, mat + ntri);
    for (size_t i = 0; i < ntri; ++i) s->tri_light.push_back(light ? light[i] : -1);
    if (normals) s->tri_n.insert(s->tri_n.end(), normals, normals + 9 * ntri);
    else s->tri_n.insert(s->tri_n.end(), 9 * ntri, 0.0f);
    static const float kDefaultUv[6] = {0.0f, 0.0f, 1.0f, 0.0f, 1.0f, 1.0f};  // Triangle::get_uvs
    if (uvs) s->tri_uv.insert(s->tri_uv.end(), uvs, uvs + 6 * ntri);
    else
        for (size_t i = 0; i < ntri; ++i) s->tri_uv.insert(s->tri_uv.end(), kDefaultUv, kDefaultUv + 6);
    uint8_t f = (uint8_t)(((flags & BG_TRI_REVERSE_ORIENTATION) ? bg::TRI_REVERSE : 0) |
                          ((flags & BG_TRI_SWAPS_HANDEDNESS) ? bg::TRI_SWAPS : 0) | (normals ? bg::TRI_NORMALS : 0));
    s->tri_flags.insert(s->tri_flags.end(), ntri, f);
    s->any_normals |= normals != nullptr && ntri > 0;
    s->any_uvs |= uvs != nullptr && ntri > 0;
    s->any_flags |= f != 0 && ntri > 0;
    return BG_OK;
}

bg_status bg_scene_add_triangles(bg_scene* s, const float* xyz, size_t ntri, const uint32_t* mat,
                                 const int32_t* light) {
    return bg_scene_add_triangle_mesh(s, xyz, ntri, mat, light, nullptr, nullptr, 0u);
}

// Image::generate_pyramid (src/io/image.rs:55-114): each level halves the previous one (at least
// 1 x 1), a texel being the mean of its 2 x 2 parents ((a + b + c + d) * 0.25 in f32).  Appends the
// levels to the scene's texels and fills ti's level table; `scale` multiplies the base image's
// channels first (Image::scale, image.rs:116-128).
static bg_status append_pyramid(bg_scene* s, const float* rgb, uint32_t w, uint32_t h, const float* scale,
                                bg::TexInfo* ti, const char* what) {
    const std::string name(what);
    if (!rgb || w == 0 || h == 0) return fail(s->ctx, BG_ERR_INVALID, name + " needs texels");
    if ((w & (w - 1)) || (h & (h - 1)))
        return fail(s->ctx, BG_ERR_UNSUPPORTED,
                    name + " sizes must be powers of two (the reference resamples other sizes with a "
                           "third-party Lanczos filter)");
    if ((uint64_t)w * h > (1ull << 28)) return fail(s->ctx, BG_ERR_INVALID, name + " too large");
    uint32_t nlev = 1;
    for (uint32_t m = std::max(w, h); m > 1; m >>= 1) ++nlev;  // 1 + ilog2(max(w, h))
    if (nlev > (uint32_t)bg::TEX_MAX_LEVELS) return fail(s->ctx, BG_ERR_INVALID, name + " too large");
    if (s->texels.size() + 2ull * w * h > 0xFFFFFFFFull) return fail(s->ctx, BG_ERR_INVALID, "too many texels");
    ti->nlevels = nlev;
    std::vector<float> cur(rgb, rgb + (size_t)w * h * 3), next;
    if (scale)
        for (size_t i = 0; i < cur.size(); ++i) cur[i] *= scale[i % 3];
    uint32_t cw = w, chh = h;
    for (uint32_t l = 0; l < nlev; ++l) {
        if (l > 0) {
            const uint32_t nw = std::max(cw / 2, 1u), nh = std::max(chh / 2, 1u);
            size_t d[4] = {0, 3, 3 * (size_t)cw, 3 * ((size_t)cw + 1)};
            if (cw == 1) {
                d[1] = 0;
                d[3] -= 3;
            }
            if (chh == 1) {
                d[2] = 0;
                d[3] -= 3 * (size_t)cw;
            }
            next.assign((size_t)nw * nh * 3, 0.0f);
            for (uint32_t y = 0; y < nh; ++y) {
                size_t src = 3 * ((size_t)(2 * y) * cw), dst = 3 * ((size_t)y * nw);
                for (uint32_t x = 0; x < nw; ++x) {
                    for (int c = 0; c < 3; ++c) {
                        next[dst] = (cur[src] + cur[src + d[1]] + cur[src + d[2]] + cur[src + d[3]]) * 0.25f;
                        ++src;
                        ++dst;
                    }
                    src += 3;
                }
            }
            cur.swap(next);
            cw = nw;
            chh = nh;
        }
        ti->lw[l] = cw;
        ti->lh[l] = chh;
        ti->loff[l] = (uint32_t)s->texels.size();
        for (size_t i = 0; i < (size_t)cw * chh; ++i)
            s->texels.push_back(make_float4(cur[3 * i], cur[3 * i + 1], cur[3 * i + 2], 0.0f));
    }
    return BG_OK;
}

bg_status bg_scene_add_texture(bg_scene* s, const bg_texture* t, uint32_t* id) {
    if (!s || !t) return BG_ERR_INVALID;
    if (!s->ctx) return BG_ERR_INVALID;
    if (s->committed) return fail(s->ctx, BG_ERR_INVALID, "scene already committed");
    if (t->kind > BG_TEXTURE_UV) return fail(s->ctx, BG_ERR_INVALID, "unknown texture kind");
    if (t->wrap > BG_WRAP_CLAMP) return fail(s->ctx, BG_ERR_INVALID, "unknown wrap mode");
    if (t->mapping > BG_MAPPING_PLANAR) return fail(s->ctx, BG_ERR_INVALID, "unknown texture mapping");
    bg::TexInfo ti{};
    ti.kind = t->kind;
    ti.wrap = t->wrap;
    ti.mapping = t->mapping;
    ti.su = t->uv_scale[0];
    ti.sv = t->uv_scale[1];
    ti.du = t->uv_delta[0];
    ti.dv = t->uv_delta[1];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) ti.m[r][c] = t->world_to_texture[4 * r + c];
    for (int k = 0; k < 3; ++k) {
        ti.vs[k] = t->vs[k];
        ti.vt[k] = t->vt[k];
    }
    ti.ds = t->ds;
    ti.dt = t->dt;
    if (t->kind == BG_TEXTURE_IMAGE) {
        bg_status st = append_pyramid(s, t->rgb, t->width, t->height, nullptr, &ti, "image texture");
        if (st != BG_OK) return st;
    }
    s->tex.push_back(ti);
    if (id) *id = (uint32_t)(s->tex.size() - 1);
    return BG_OK;
}

// InfiniteAreaLight::new (src/lights/infinite.rs:38-80), the image part: the environment map scaled
// by the intensity, as a MIPMap with repeat wrapping.  The sampling distribution and the world's
// bounding sphere wait for the commit, which knows the scene's bounds.
bg_status bg_scene_add_infinite_light(bg_scene* s, const bg_infinite_light* l) {
    if (!s || !l) return BG_ERR_INVALID;
    if (!s->ctx) return BG_ERR_INVALID;
    if (s->committed) return fail(s->ctx, BG_ERR_INVALID, "scene already committed");
    if (s->has_inf) return fail(s->ctx, BG_ERR_UNSUPPORTED, "a scene holds at most one infinite light");
    for (int k = 0; k < 3; ++k)
        if (!std::isfinite(l->intensity[k])) return fail(s->ctx, BG_ERR_INVALID, "infinite light intensity is not finite");
    for (int k = 0; k < 12; ++k)
        if (!std::isfinite(l->light_to_world[k]))
            return fail(s->ctx, BG_ERR_INVALID, "infinite light transform is not finite");
    const float* m = l->light_to_world;
    const float det = m[0] * (m[5] * m[10] - m[6] * m[9]) - m[1] * (m[4] * m[10] - m[6] * m[8]) +
                      m[2] * (m[4] * m[9] - m[5] * m[8]);
    if (!(det != 0.0f) || !std::isfinite(det))
        return fail(s->ctx, BG_ERR_INVALID, "infinite light transform is singular");
    if (l->rgb && l->width && l->height && (uint64_t)l->width * l->height <= (1ull << 28)) {
        const size_t nf = 3 * (size_t)l->width * l->height;
        for (size_t i = 0; i < nf; ++i)
            if (!(l->rgb[i] >= 0.0f) || !std::isfinite(l->rgb[i]))
                return fail(s->ctx, BG_ERR_INVALID,
                            "environment map texels must be finite and >= 0 (its sampling distribution is a CDF)");
    }
    bg::TexInfo ti{};
    ti.kind = BG_TEXTURE_IMAGE;
    ti.wrap = BG_WRAP_REPEAT;
    const size_t texels0 = s->texels.size();
    bg_status st = append_pyramid(s, l->rgb, l->width, l->height, l->intensity, &ti, "environment map");
    if (st != BG_OK) {
        s->texels.resize(texels0);
        return st;
    }
    s->inf_map = ti;
    std::memcpy(s->inf_l2w, l->light_to_world, sizeof(s->inf_l2w));
    bgi::affine_inverse(l->light_to_world, s->inf_w2l);
    s->has_inf = true;
    return BG_OK;
}

bg_status bg_scene_add_spheres(bg_scene* s, const bg_sphere* sp, size_t n) {
    if (!s || (n && !sp)) return BG_ERR_INVALID;
    if (!s->ctx) return BG_ERR_INVALID;
    if (s->committed) return fail(s->ctx, BG_ERR_INVALID, "scene already committed");
    for (size_t i = 0; i < n; ++i) {
        if (sp[i].material_id >= s->mats.size()) return fail(s->ctx, BG_ERR_INVALID, "sphere has an unknown material id");
        if (sp[i].light_id >= (int32_t)s->lights.size())
            return fail(s->ctx, BG_ERR_INVALID, "sphere has an unknown area light id");
        if (!(sp[i].radius > 0.0f) || !std::isfinite(sp[i].radius))
            return fail(s->ctx, BG_ERR_INVALID, "sphere radius must be finite and > 0");
    }
    s->sph.insert(s->sph.end(), sp, sp + n);
    return BG_OK;
}

bg_status bg_scene_add_quadrics(bg_scene* s, const bg_quadric* q, size_t n) {
    if (!s || (n && !q)) return BG_ERR_INVALID;
    if (!s->ctx) return BG_ERR_INVALID;
    if (s->committed) return fail(s->ctx, BG_ERR_INVALID, "scene already committed");
    for (size_t i = 0; i < n; ++i) {
        if (q[i].kind > BG_QUADRIC_CONE) return fail(s->ctx, BG_ERR_INVALID, "unknown quadric kind");
        if (q[i].material_id >= s->mats.size()) return fail(s->ctx, BG_ERR_INVALID, "quadric has an unknown material id");
        if (q[i].light_id >= (int32_t)s->lights.size())
            return fail(s->ctx, BG_ERR_INVALID, "quadric has an unknown area light id");
        if (q[i].light_id >= 0 && q[i].kind == BG_QUADRIC_CONE)
            return fail(s->ctx, BG_ERR_UNSUPPORTED, "cones cannot be area lights (the reference's Cone has no sample())");
        if (!(q[i].radius > 0.0f) || !std::isfinite(q[i].radius))
            return fail(s->ctx, BG_ERR_INVALID, "quadric radius must be finite and > 0");
        if (q[i].kind == BG_QUADRIC_CONE && !(q[i].height != 0.0f))
            return fail(s->ctx, BG_ERR_INVALID, "cone height must be non-zero");
        for (int k = 0; k < 12; ++k)
            if (!std::isfinite(q[i].object_to_world[k]) || !std::isfinite(q[i].world_to_object[k]))
                return fail(s->ctx, BG_ERR_INVALID, "quadric transform is not finite");
    }
    s->quads.insert(s->quads.end(), q, q + n);
    return BG_OK;
}

// ---- the infinite light's sampling distribution, built on the host at commit
namespace {
int32_t sat_i32(float f) {  // `as i32`: saturating, NaN to 0
    if (std::isnan(f)) return 0;
    if (f >= 2147483648.0f) return 2147483647;
    if (f <= -2147483648.0f) return (-2147483647 - 1);
    return (int32_t)f;
}
int32_t imod(int32_t a, int32_t b) {  // math::modulo (math.rs:43-50)
    int32_t r = a - (a / b) * b;
    return r < 0 ? r + b : r;
}
// Image::get_channel with repeat wrapping (image.rs:130-159), the three channels.
void env_texel(const bg_scene* s, const bg::TexInfo& t, int level, int32_t x, int32_t y, float out[3]) {
    const int32_t w = (int32_t)t.lw[level], h = (int32_t)t.lh[level];
    x = imod(x, w);
    y = imod(y, h);
    const float4 v = s->texels[t.loff[level] + (size_t)y * (size_t)w + (size_t)x];
    out[0] = v.x;
    out[1] = v.y;
    out[2] = v.z;
}
// MIPMap::triangle (mipmap.rs:156-173)
void env_bilerp(const bg_scene* s, const bg::TexInfo& t, int level, float s0, float t0, float out[3]) {
    const float fs = s0 * (float)t.lw[level] - 0.5f, ft = t0 * (float)t.lh[level] - 0.5f;
    const float ds = fs - std::floor(fs), dt = ft - std::floor(ft);
    const int32_t x = sat_i32(std::floor(fs)), y = sat_i32(std::floor(ft));
    const int32_t x1 = (int32_t)((uint32_t)x + 1u), y1 = (int32_t)((uint32_t)y + 1u);
    float a[3], b[3], c[3], d[3];
    env_texel(s, t, level, x, y, a);
    env_texel(s, t, level, x, y1, b);
    env_texel(s, t, level, x1, y, c);
    env_texel(s, t, level, x1, y1, d);
    const float wa = (1.0f - ds) * (1.0f - dt), wb = (1.0f - ds) * dt, wc = ds * (1.0f - dt), wd = ds * dt;
    for (int k = 0; k < 3; ++k) out[k] = wa * a[k] + wb * b[k] + wc * c[k] + wd * d[k];
}
// MIPMap::trilinear_filter (mipmap.rs:46-63)
void env_trilinear(const bg_scene* s, const bg::TexInfo& t, float s0, float t0, float width, float out[3]) {
    const float top = (float)(t.nlevels - 1);
    const float level = top + std::log2(std::fmax(width, 1e-8f));
    if (level < 0.0f) return env_bilerp(s, t, 0, s0, t0, out);
    if (level >= top) return env_texel(s, t, (int)t.nlevels - 1, 0, 0, out);
    const int il = (int)std::floor(level);
    const float f = level - std::floor(level);
    float a[3], b[3];
    env_bilerp(s, t, il, s0, t0, a);
    env_bilerp(s, t, il + 1, s0, t0, b);
    for (int k = 0; k < 3; ++k) out[k] = (1.0f - f) * a[k] + f * b[k];
}
// find_interval (math.rs:70-87) over a cdf of `size` entries.
uint32_t cdf_find_interval(const float* cdf, uint32_t size, float u) {
    uint32_t first = 0, len = size;
    while (len > 0) {
        const uint32_t half = len >> 1, middle = first + half;
        if (cdf[middle] <= u) {
            first = middle + 1;
            len -= half + 1;
        } else {
            len = half;
        }
    }
    const int64_t r = (int64_t)first - 1;
    return (uint32_t)(r < 0 ? 0 : (r > (int64_t)size - 2 ? (int64_t)size - 2 : r));
}
// Guide table of a cdf of n + 1 entries: g + 1 entries, entry k = find_interval at u = k / g.
void cdf_guide(const float* cdf, uint32_t n, uint32_t g, uint32_t* out) {
    for (uint32_t k = 0; k <= g; ++k) out[k] = cdf_find_interval(cdf, n + 1, (float)k / (float)g);
}
// Buckets for n intervals: a power of two near n / 8, at least 1.
uint32_t guide_buckets(uint32_t n) {
    uint32_t g = 1;
    while (g * 16 <= n) g *= 2;
    return g;
}
// Distribution1D::new (sampling.rs:22-47) over func[0..n): cdf has n + 1 entries.
float dist1d_build(const float* func, uint32_t n, float* cdf) {
    cdf[0] = 0.0f;
    for (uint32_t i = 1; i <= n; ++i) cdf[i] = cdf[i - 1] + func[i - 1] / (float)n;
    const float func_int = cdf[n];
    if (func_int == 0.0f) {
        for (uint32_t i = 1; i <= n; ++i) cdf[i] = (float)i / (float)n;
    } else {
        for (uint32_t i = 1; i <= n; ++i) cdf[i] /= func_int;
    }
    return func_int;
}
}  // namespace

// InfiniteAreaLight::new (infinite.rs:38-80), the part that needs the scene: the luminance of the
// map over a 2w x 2h grid weighted by sin(theta), its Distribution2D (sampling.rs:79-97) and the
// world's bounding sphere (Bounds3::bounding_sphere, bounds3.rs:208-215).
static bg_status commit_infinite_light(bg_scene* s, bg::InfLight* L) {
    bg_ctx* ctx = s->ctx;
    const bg::TexInfo& map = s->inf_map;
    const uint32_t nu = 2 * map.lw[0], nv = 2 * map.lh[0];
    const float PI = 3.14159265358979323846f;
    const float fwidth = 0.5f / (float)std::min(nu, nv);
    std::vector<float> func((size_t)nu * nv), cond_cdf((size_t)nv * (nu + 1)), cond_int(nv), marg_cdf(nv + 1);
    for (uint32_t v = 0; v < nv; ++v) {
        const float vp = ((float)v + 0.5f) / (float)nv;
        const float sin_theta = std::sin(PI * ((float)v + 0.5f) / (float)nv);
        for (uint32_t u = 0; u < nu; ++u) {
            const float up = ((float)u + 0.5f) / (float)nu;
            float c[3];
            env_trilinear(s, map, up, vp, fwidth, c);
            const float y = 0.212671f * c[0] + 0.715160f * c[1] + 0.072169f * c[2];  // RGBSpectrum::y
            func[(size_t)v * nu + u] = y * sin_theta;
        }
    }
    for (uint32_t v = 0; v < nv; ++v)
        cond_int[v] = dist1d_build(&func[(size_t)v * nu], nu, &cond_cdf[(size_t)v * (nu + 1)]);
    const float marg_int = dist1d_build(cond_int.data(), nv, marg_cdf.data());
    *L = bg::InfLight{};
    L->map = map;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) {
            L->l2w[r][c] = s->inf_l2w[4 * r + c];
            L->w2l[r][c] = s->inf_w2l[4 * r + c];
        }
    float center[3], radius = 0.0f;
    bool inside = true;
    for (int k = 0; k < 3; ++k) {
        center[k] = (s->bmin[k] + s->bmax[k]) * (1.0f / 2.0f);
        inside = inside && center[k] >= s->bmin[k] && center[k] <= s->bmax[k];
    }
    if (inside) {
        const float dx = center[0] - s->bmax[0], dy = center[1] - s->bmax[1], dz = center[2] - s->bmax[2];
        radius = std::sqrt(dx * dx + dy * dy + dz * dz);
    }
    std::memcpy(L->center, center, sizeof(center));
    L->radius = radius;
    L->nu = nu;
    L->nv = nv;
    L->marg_int = marg_int;
    L->gu = guide_buckets(nu);
    L->gv = guide_buckets(nv);
    std::vector<uint32_t> cond_guide((size_t)nv * (L->gu + 1)), marg_guide(L->gv + 1);
    for (uint32_t v = 0; v < nv; ++v)
        cdf_guide(&cond_cdf[(size_t)v * (nu + 1)], nu, L->gu, &cond_guide[(size_t)v * (L->gu + 1)]);
    cdf_guide(marg_cdf.data(), nv, L->gv, marg_guide.data());
    bg_status st;
    if ((st = upload(ctx, cond_cdf, &L->cond_cdf, &s->allocs)) != BG_OK) return st;
    if ((st = upload(ctx, func, &L->cond_func, &s->allocs)) != BG_OK) return st;
    if ((st = upload(ctx, cond_int, &L->cond_int, &s->allocs)) != BG_OK) return st;
    if ((st = upload(ctx, marg_cdf, &L->marg_cdf, &s->allocs)) != BG_OK) return st;
    if ((st = upload(ctx, cond_int, &L->marg_func, &s->allocs)) != BG_OK) return st;
    if ((st = upload(ctx, cond_guide, &L->cond_guide, &s->allocs)) != BG_OK) return st;
    if ((st = upload(ctx, marg_guide, &L->marg_guide, &s->allocs)) != BG_OK) return st;
    CK(cudaStreamSynchronize(ctx->stream));  // the host vectors end here
    return BG_OK;
}

bg_status bg_scene_commit(bg_scene* s, uint32_t kind, bg_build_stats* stats) {
    if (!s) return BG_ERR_INVALID;
    if (!s->ctx) return BG_ERR_INVALID;
    bg_ctx* ctx = s->ctx;
    if (s->committed) return fail(ctx, BG_ERR_INVALID, "scene already committed");
    if (kind > BG_BVH_WIDE2) return fail(ctx, BG_ERR_INVALID, "unknown BVH kind");
    auto t0 = std::chrono::steady_clock::now();
    CK(cudaSetDevice(ctx->device));
    const uint32_t ntri = (uint32_t)s->tri_mat.size(), nsph = (uint32_t)s->sph.size();
    const uint32_t nquad = (uint32_t)s->quads.size();
    bg::HostPrims hp{s->tri.data(), ntri, s->sph.data(), nsph, s->quads.data(), nquad};
    {
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t i = 0; i < hp.count(); ++i) {
            float bl[3], bh[3];
            bg::prim_bounds(hp, i, bl, bh);
            for (int k = 0; k < 3; ++k) {
                lo[k] = std::fmin(lo[k], bl[k]);
                hi[k] = std::fmax(hi[k], bh[k]);
            }
        }
        for (int k = 0; k < 3; ++k) {
            s->bmin[k] = hp.count() ? lo[k] : 0.0f;
            s->bmax[k] = hp.count() ? hi[k] : 0.0f;
        }
    }
    // triangles as float4 triplets with material / emission / light-index tags
    std::vector<float4> tri4(3 * (size_t)ntri);
    std::vector<uint32_t> light_prims;
    for (uint32_t i = 0; i < ntri; ++i) {
        const float* v = &s->tri[9 * (size_t)i];
        int32_t li = -1;
        if (s->tri_light[i] >= 0) {
            li = (int32_t)light_prims.size();
            light_prims.push_back(i);
        }
        uint32_t m = s->tri_mat[i];
        int32_t e = s->tri_light[i];
        float4 a = make_float4(v[0], v[1], v[2], 0.0f), b = make_float4(v[3], v[4], v[5], 0.0f),
               c = make_float4(v[6], v[7], v[8], 0.0f);
        std::memcpy(&a.w, &m, 4);
        std::memcpy(&b.w, &e, 4);
        std::memcpy(&c.w, &li, 4);
        tri4[3 * i] = a;
        tri4[3 * i + 1] = b;
        tri4[3 * i + 2] = c;
    }
    std::vector<float4> sph4(nsph);
    std::vector<uint32_t> sph_mat(nsph);
    for (uint32_t i = 0; i < nsph; ++i) {
        sph4[i] = make_float4(s->sph[i].center[0], s->sph[i].center[1], s->sph[i].center[2], s->sph[i].radius);
        sph_mat[i] = s->sph[i].material_id;
    }
    // quadric records: o2w rows, w2o rows (o2w itself when it is the identity, cylinder.rs:37-41),
    // (radius, inner, z_min, z_max), (height, phi_max, flags, material)
    std::vector<float4> quad4((size_t)bg::QUADRIC_F4 * nquad);
    for (uint32_t i = 0; i < nquad; ++i) {
        const bg_quadric& q = s->quads[i];
        float4* r = &quad4[(size_t)bg::QUADRIC_F4 * i];
        bool ident = true;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 4; ++b) ident &= q.object_to_world[4 * a + b] == ((a == b) ? 1.0f : 0.0f);
        const float* w2o = ident ? q.object_to_world : q.world_to_object;
        for (int a = 0; a < 3; ++a) {
            r[a] = make_float4(q.object_to_world[4 * a], q.object_to_world[4 * a + 1], q.object_to_world[4 * a + 2],
                               q.object_to_world[4 * a + 3]);
            r[3 + a] = make_float4(w2o[4 * a], w2o[4 * a + 1], w2o[4 * a + 2], w2o[4 * a + 3]);
        }
        const float* m = q.object_to_world;  // Transform::swaps_handedness (transform.rs:212-218)
        float det = m[0] * (m[5] * m[10] - m[6] * m[9]) - m[1] * (m[4] * m[10] - m[6] * m[8]) +
                    m[2] * (m[4] * m[9] - m[5] * m[8]);
        uint32_t flags = q.kind | ((q.reverse_orientation ? 1u : 0u) << 8) | ((det < 0.0f ? 1u : 0u) << 9);
        float phi_max = std::fmin(std::fmax(q.phi_max_deg, 0.0f), 360.0f) * (3.14159265358979323846f / 180.0f);
        r[6] = make_float4(q.radius, q.inner_radius, std::fmin(q.z_min, q.z_max), std::fmax(q.z_min, q.z_max));
        float fbits, mbits;
        std::memcpy(&fbits, &flags, 4);
        std::memcpy(&mbits, &q.material_id, 4);
        r[7] = make_float4(q.height, phi_max, fbits, mbits);
    }
    std::vector<bg::Material> mats(s->mats.size());
    for (size_t i = 0; i < mats.size(); ++i) {
        const bg_material& m = s->mats[i];
        bg::Material& d = mats[i];
        d.type = m.type;
        std::memcpy(d.kd, m.kd, sizeof(d.kd));
        std::memcpy(d.ks, m.ks, sizeof(d.ks));
        float a = m.roughness;
        if (m.type == BG_MAT_PLASTIC && m.remap_roughness) a = roughness_to_alpha(a);
        d.alpha = std::fmax(a, 0.001f);  // TrowbridgeReitzDistribution::new (microfacet.rs:38-43)
        std::memcpy(d.eta, m.eta, sizeof(d.eta));
        std::memcpy(d.k, m.k, sizeof(d.k));
        d.ior = m.ior;
        // MatteMaterial: sigma clamped to [0, 90], OrenNayer::new's A and B (oren_nayer.rs:20-30)
        d.sigma = m.type == BG_MAT_MATTE ? std::fmin(std::fmax(m.sigma, 0.0f), 90.0f) : 0.0f;
        const float sr = d.sigma * (3.14159265358979323846f / 180.0f);  // f32::to_radians
        const float s2 = sr * sr;
        d.on_a = 1.0f - (s2 / (2.0f * (s2 + 0.33f)));
        d.on_b = 0.45f * s2 / (s2 + 0.09f);
        d.kd_tex = (m.type == BG_MAT_MATTE || m.type == BG_MAT_PLASTIC) ? m.kd_texture : 0u;
        d.ks_tex = m.type == BG_MAT_PLASTIC ? m.ks_texture : 0u;
        if (d.kd_tex > s->tex.size() || d.ks_tex > s->tex.size())
            return fail(ctx, BG_ERR_INVALID, "material " + std::to_string(i) + " refers to an unknown texture");
        d.pad = 0;
    }
    std::vector<bg::Emission> emis(s->lights.size());
    for (size_t i = 0; i < emis.size(); ++i) {
        std::memcpy(emis[i].intensity, s->lights[i].intensity, sizeof(emis[i].intensity));
        emis[i].two_sided = s->lights[i].two_sided;
    }
    // the light list: emitting triangles, spheres and quadrics in order, then the infinite light
    std::vector<int32_t> sph_emis(nsph, -1), quad_emis(nquad, -1);
    bool any_sph_light = false, any_quad_light = false;
    for (uint32_t i = 0; i < nsph; ++i)
        if (s->sph[i].light_id >= 0) {
            sph_emis[i] = s->sph[i].light_id;
            light_prims.push_back(ntri + i);
            any_sph_light = true;
        }
    for (uint32_t i = 0; i < nquad; ++i)
        if (s->quads[i].light_id >= 0) {
            quad_emis[i] = s->quads[i].light_id;
            light_prims.push_back(ntri + nsph + i);
            any_quad_light = true;
        }
    if (s->has_inf) light_prims.push_back(bg::LIGHT_INFINITE);
    bg::Scene& d = s->dev;
    d = bg::Scene{};
    d.ntri = ntri;
    d.nsph = nsph;
    d.nquad = nquad;
    d.nlights = (uint32_t)light_prims.size();
    bg_status st;
    if ((st = upload(ctx, quad4, &d.quads, &s->allocs)) != BG_OK) return st;
    if ((st = upload(ctx, tri4, &d.tri, &s->allocs)) != BG_OK) return st;
    if ((st = upload(ctx, sph4, &d.sph, &s->allocs)) != BG_OK) return st;
    if ((st = upload(ctx, sph_mat, &d.sph_mat, &s->allocs)) != BG_OK) return st;
    if ((st = upload(ctx, mats, &d.mats, &s->allocs)) != BG_OK) return st;
    if ((st = upload(ctx, emis, &d.emis, &s->allocs)) != BG_OK) return st;
    if ((st = upload(ctx, light_prims, &d.light_prims, &s->allocs)) != BG_OK) return st;
    {   // the material class of every primitive, for the binning pass (one byte each instead of the
        // primitive's 16-byte record and its material)
        std::vector<uint8_t> cls((size_t)ntri + nsph + nquad);
        for (uint32_t i = 0; i < ntri; ++i) cls[i] = (uint8_t)mats[s->tri_mat[i]].type;
        for (uint32_t i = 0; i < nsph; ++i) cls[ntri + i] = (uint8_t)mats[sph_mat[i]].type;
        for (uint32_t i = 0; i < nquad; ++i) cls[ntri + nsph + i] = (uint8_t)mats[s->quads[i].material_id].type;
        if (!cls.empty() && (st = upload(ctx, cls, &d.prim_cls, &s->allocs)) != BG_OK) return st;
    }
    if (any_sph_light && (st = upload(ctx, sph_emis, &d.sph_emis, &s->allocs)) != BG_OK) return st;
    if (any_quad_light && (st = upload(ctx, quad_emis, &d.quad_emis, &s->allocs)) != BG_OK) return st;
    if (s->any_normals || s->any_flags) {
        std::vector<uint8_t> flags;
        std::string why;
        if (!bgi::triangle_light_sides(s, &flags, &why)) return fail(ctx, BG_ERR_UNSUPPORTED, why);
        if ((st = upload(ctx, flags, &d.tri_flags, &s->allocs)) != BG_OK) return st;
    }
    if (s->any_normals) {
        std::vector<float4> ns(3 * (size_t)ntri);
        for (size_t k = 0; k < ns.size(); ++k)
            ns[k] = make_float4(s->tri_n[3 * k], s->tri_n[3 * k + 1], s->tri_n[3 * k + 2], 0.0f);
        if ((st = upload(ctx, ns, &d.tri_ns, &s->allocs)) != BG_OK) return st;
    }
    if (s->any_uvs) {
        std::vector<float2> uv(3 * (size_t)ntri);
        for (size_t k = 0; k < uv.size(); ++k) uv[k] = make_float2(s->tri_uv[2 * k], s->tri_uv[2 * k + 1]);
        if ((st = upload(ctx, uv, &d.tri_uv, &s->allocs)) != BG_OK) return st;
    }
    if (!s->tex.empty()) {
        if ((st = upload(ctx, s->tex, &d.tex, &s->allocs)) != BG_OK) return st;
        d.ntex = (uint32_t)s->tex.size();
    }
    if (!s->texels.empty())
        if ((st = upload(ctx, s->texels, &d.texels, &s->allocs)) != BG_OK) return st;
    uint64_t inf_bytes = 0;
    if (s->has_inf) {
        std::vector<bg::InfLight> inf(1);
        if ((st = commit_infinite_light(s, &inf[0])) != BG_OK) return st;
        if ((st = upload(ctx, inf, &d.inf, &s->allocs)) != BG_OK) return st;
        const uint64_t nu = inf[0].nu, nv = inf[0].nv;
        inf_bytes = sizeof(bg::InfLight) + 4 * (nv * (nu + 1) + nu * nv + 2 * nv + nv + 1) +
                    4 * (nv * ((uint64_t)inf[0].gu + 1) + inf[0].gv + 1);
    }
    uint64_t nodes = 0;
    if (kind == BG_BVH_WIDE) {
        bg::Bvh8 b;
        bg::build_bvh8(hp, &b);
        // nodes and leaf primitives in one allocation: the range traversal reads, which an L2
        // access-policy window can keep resident (BG_TUNE_L2_PERSIST)
        const size_t nb = (b.nodes.size() * sizeof(bg::Bvh8Node) + 255) & ~(size_t)255;
        const size_t lb = b.leaf_prims.size() * sizeof(float4);
        void* hot = nullptr;
        if ((st = dalloc(ctx, nb + lb, &hot, &s->allocs)) != BG_OK) return st;
        if (!b.nodes.empty())
            CK(cudaMemcpyAsync(hot, b.nodes.data(), b.nodes.size() * sizeof(bg::Bvh8Node), cudaMemcpyHostToDevice,
                               ctx->stream));
        if (lb) CK(cudaMemcpyAsync((char*)hot + nb, b.leaf_prims.data(), lb, cudaMemcpyHostToDevice, ctx->stream));
        d.nodes8 = (const bg::Bvh8Node*)hot;
        d.leaf_prims = (const float4*)((char*)hot + nb);
        s->hot = hot;
        s->hot_bytes = nb + lb;
        d.n_nodes8 = (uint32_t)b.nodes.size();
        nodes = b.nodes.size();
    } else if (kind == BG_BVH_WIDE2) {
        bg::Bvh2 b;
        bg::build_bvh2(hp, &b, 0);
        if ((st = upload(ctx, b.nodes, (const bg::Bvh2Node**)&d.nodes, &s->allocs)) != BG_OK) return st;
        if ((st = upload(ctx, b.leaf_prims, &d.leaf_prims, &s->allocs)) != BG_OK) return st;
        d.n_nodes = (uint32_t)b.nodes.size();
        nodes = b.nodes.size();
    } else {
        bg::RefBvh r;
        if (!bg::build_reference_bvh(hp, kind == BG_BVH_REFERENCE, &r, kFaithfulMaxPrims))
            return fail(ctx, BG_ERR_UNSUPPORTED,
                        "the reference's chain-shaped BVH build is limited to " + std::to_string(kFaithfulMaxPrims) +
                            " primitives; use BG_BVH_REFERENCE_FIXED");
        if ((st = upload(ctx, r.nodes, &d.ref_nodes, &s->allocs)) != BG_OK) return st;
        if ((st = upload(ctx, r.order, &d.ref_order, &s->allocs)) != BG_OK) return st;
        d.ref_nnodes = (uint32_t)r.nodes.size();
        nodes = r.nodes.size();
    }
    CK(cudaStreamSynchronize(ctx->stream));
    s->kind = kind;
    s->committed = true;
    if (stats) {
        stats->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        stats->nodes = nodes;
        stats->prims = (uint64_t)ntri + nsph + nquad;
        const bool wide = kind == BG_BVH_WIDE || kind == BG_BVH_WIDE2;
        uint64_t bytes = tri4.size() * 16 + sph4.size() * 16 +
                         nodes * (kind == BG_BVH_WIDE ? 80 : (kind == BG_BVH_WIDE2 ? 64 : 32)) +
                         ((uint64_t)ntri + nsph + nquad) * (wide ? 48 : 4) + quad4.size() * 16 +
                         ((s->any_normals || s->any_flags) ? (uint64_t)ntri : 0) +
                         (s->any_normals ? 48ull * ntri : 0) + (s->any_uvs ? 24ull * ntri : 0) +
                         s->tex.size() * sizeof(bg::TexInfo) + s->texels.size() * 16 + inf_bytes;
        stats->device_bytes = bytes;
    }
    return BG_OK;
}

// ---------------------------------------------------------------- ray queries
static bg_status trace_device(bg_ctx* ctx, const bg_scene* s, const bg_ray* d_rays, size_t n, bg_hit* d_hits,
                              uint8_t* d_occ, bool any, float* ms) {
    if (!ctx || !s || !s->committed || s->ctx != ctx) return fail(ctx, BG_ERR_INVALID, "scene not committed on this context");
    if (n >= (1ull << 31)) return fail(ctx, BG_ERR_INVALID, "too many rays");
    CK(cudaSetDevice(ctx->device));
    if (n == 0) {
        if (ms) *ms = 0.0f;
        return BG_OK;
    }
    CK(cudaEventRecord(ctx->ev_begin, ctx->stream));
    const bool ref_layout = s->kind == BG_BVH_REFERENCE || s->kind == BG_BVH_REFERENCE_FIXED;
    bg::launch_trace(s->dev, ref_layout, any, d_rays, n, d_hits, d_occ, ctx->d_err, nullptr, ctx->d_head,
                     ctx->shape, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev_end, ctx->stream));
    bg_status st = check_device_error(ctx, nullptr);
    if (st != BG_OK) return st;
    if (ms) CK(cudaEventElapsedTime(ms, ctx->ev_begin, ctx->ev_end));
    return BG_OK;
}

bg_status bg_trace_closest_device(bg_ctx* ctx, const bg_scene* s, const bg_ray* d_rays, size_t n, bg_hit* d_hits,
                                  float* ms) {
    if (!ctx || (n && (!d_rays || !d_hits))) return BG_ERR_INVALID;
    return trace_device(ctx, s, d_rays, n, d_hits, nullptr, false, ms);
}
bg_status bg_trace_any_device(bg_ctx* ctx, const bg_scene* s, const bg_ray* d_rays, size_t n, uint8_t* d_occ,
                              float* ms) {
    if (!ctx || (n && (!d_rays || !d_occ))) return BG_ERR_INVALID;
    return trace_device(ctx, s, d_rays, n, nullptr, d_occ, true, ms);
}

static bg_status trace_host(bg_ctx* ctx, const bg_scene* s, const bg_ray* rays, size_t n, void* out, bool any) {
    if (!ctx || !s || (n && (!rays || !out))) return BG_ERR_INVALID;
    if (n == 0) return BG_OK;
    CK(cudaSetDevice(ctx->device));
    void *dr = nullptr, *dh = nullptr;
    std::vector<void*> tmp;
    bg_status st = dalloc(ctx, n * sizeof(bg_ray), &dr, &tmp);
    if (st == BG_OK) st = dalloc(ctx, n * (any ? 1 : sizeof(bg_hit)), &dh, &tmp);
    if (st == BG_OK) {
        cudaError_t e = cudaMemcpyAsync(dr, rays, n * sizeof(bg_ray), cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) st = cuda_fail(ctx, e, "cudaMemcpyAsync");
    }
    if (st == BG_OK) st = trace_device(ctx, s, (const bg_ray*)dr, n, any ? nullptr : (bg_hit*)dh,
                                       any ? (uint8_t*)dh : nullptr, any, nullptr);
    if (st == BG_OK) {
        cudaError_t e = cudaMemcpyAsync(out, dh, n * (any ? 1 : sizeof(bg_hit)), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) st = cuda_fail(ctx, e, "cudaMemcpyAsync");
    }
    cudaStreamSynchronize(ctx->stream);
    dfree_all(ctx, tmp);
    return st;
}

bg_status bg_trace_closest(bg_ctx* ctx, const bg_scene* s, const bg_ray* rays, size_t n, bg_hit* hits) {
    return trace_host(ctx, s, rays, n, hits, false);
}
bg_status bg_trace_any(bg_ctx* ctx, const bg_scene* s, const bg_ray* rays, size_t n, uint8_t* occ) {
    return trace_host(ctx, s, rays, n, occ, true);
}

// ---------------------------------------------------------------- render
extern "C++" {
void bgi::scene_bounds(const bg_scene* s, float lo[3], float inv[3]) {
    for (int k = 0; k < 3; ++k) {
        const float ext = std::fmax(s->bmax[k] - s->bmin[k], 1e-6f) * 1.002f;
        lo[k] = s->bmin[k] - 0.001f * ext;
        inv[k] = 1.0f / ext;
    }
}

bg_status bgi::validate_render(bg_ctx* ctx, const bg_scene* s, const bg_camera* cam, const bg_render_opts* o,
                               const float* rgb_out) {
    if (!ctx || !s || !cam || !o) return BG_ERR_INVALID;
    if (!s->committed || s->ctx != ctx) return fail(ctx, BG_ERR_INVALID, "scene not committed on this context");
    if (cam->width == 0 || cam->height == 0 || (uint64_t)cam->width * cam->height >= (1ull << 31))
        return fail(ctx, BG_ERR_INVALID, "bad film resolution");
    if (!(cam->lens_radius >= 0.0f) || !std::isfinite(cam->lens_radius))
        return fail(ctx, BG_ERR_INVALID, "lens_radius must be finite and >= 0");
    if (cam->lens_radius > 0.0f && (!(cam->focal_distance > 0.0f) || !std::isfinite(cam->focal_distance)))
        return fail(ctx, BG_ERR_INVALID, "a thin-lens camera needs a finite focal_distance > 0");
    if (!(cam->fov_deg > 0.0f && cam->fov_deg < 180.0f)) return fail(ctx, BG_ERR_INVALID, "fov out of range");
    if (o->mode > BG_MODE_PBRT) return fail(ctx, BG_ERR_INVALID, "unknown mode");
    if (o->mode == BG_MODE_REF_COMPAT && (s->kind == BG_BVH_WIDE || s->kind == BG_BVH_WIDE2))
        return fail(ctx, BG_ERR_INVALID, "REF_COMPAT rendering needs a BG_BVH_REFERENCE* scene layout");
    if (o->max_depth > 250) return fail(ctx, BG_ERR_INVALID, "max_depth must be <= 250");
    if (o->integrator > BG_INTEGRATOR_DIRECT) return fail(ctx, BG_ERR_INVALID, "unknown integrator");
    if (o->light_strategy > BG_LIGHT_UNIFORM_ONE) return fail(ctx, BG_ERR_INVALID, "unknown light strategy");
    if (o->integrator != BG_INTEGRATOR_PATH && o->max_depth > bg::TREE_MAX_DEPTH)
        return fail(ctx, BG_ERR_INVALID, "the Whitted and direct-lighting integrators accept max_depth <= 30");
    bg::StratParams sp;
    if (const char* why = bg::strat_params(o->sampler, o->spp, o->x_pixel_samples, o->y_pixel_samples,
                                           o->sampled_dimensions, o->jitter_samples, &sp))
        return fail(ctx, BG_ERR_INVALID, why);
    if (o->integrator != BG_INTEGRATOR_PATH && sp.dims > 1)
        return fail(ctx, BG_ERR_UNSUPPORTED,
                    "the Whitted and direct-lighting integrators take sampled_dimensions <= 1 (the camera sample): "
                    "the reference's later calls follow its depth-first recursion");
    if (!(o->flags & BG_RENDER_NO_READBACK) && !rgb_out) return BG_ERR_INVALID;
    return BG_OK;
}
}  // extern "C++"

bg_status bg_render(bg_ctx* ctx, const bg_scene* s, const bg_camera* cam, const bg_render_opts* o, float* rgb_out,
                    bg_render_stats* stats) {
    bg_status st = validate_render(ctx, s, cam, o, rgb_out);
    if (st != BG_OK) return st;
    CK(cudaSetDevice(ctx->device));
    if ((st = ensure_film(ctx, cam->width, cam->height)) != BG_OK) return st;
    if (!(o->flags & BG_RENDER_ACCUMULATE)) {
        bg::launch_clear_film(ctx->film, ctx->stream);
        CK(cudaMemsetAsync(ctx->film.nan_count, 0, sizeof(unsigned long long), ctx->stream));
    }
    bg::Camera dc = make_camera(*cam);
    bg::RenderParams rp{cam->width, cam->height, o->spp, o->max_depth, o->first_sample, o->rr_threshold, o->seed,
                        {0, 0, 0}, {0, 0, 0}};
    scene_bounds(s, rp.bmin, rp.binv);
    rp = bg::with_camera(rp, dc, o->spp);
    bg::strat_params(o->sampler, o->spp, o->x_pixel_samples, o->y_pixel_samples, o->sampled_dimensions,
                     o->jitter_samples, &rp.strat);  // checked by validate_render
    rp.pixel_tiles = ctx->shape.tile_pixels ? 1u : 0u;
    const uint64_t npix = (uint64_t)cam->width * cam->height;
    const uint64_t total = npix * o->spp;
    uint64_t launches = 0;
    const bool tree = o->integrator != BG_INTEGRATOR_PATH;
    bool wavefront = !tree && (o->mode == BG_MODE_PBRT && (s->kind == BG_BVH_WIDE || s->kind == BG_BVH_WIDE2));
    uint32_t cap = 0;
    if (wavefront) {
        cap = (uint32_t)std::min<uint64_t>(ctx->max_queue, std::max<uint64_t>(total, 1));
        if ((st = ensure_wave(ctx, cap)) != BG_OK) return st;
    }
    const bool timing = wavefront && (o->flags & BG_RENDER_STAGE_TIMING);
    const uint64_t nwaves = wavefront ? (total + cap - 1) / cap : 0;
    const size_t ev_per_wave = 4 * ((size_t)o->max_depth + 1);
    if (timing) {
        while (ctx->timing_ev.size() < nwaves * ev_per_wave) {
            cudaEvent_t e;
            CK(cudaEventCreate(&e));
            ctx->timing_ev.push_back(e);
        }
    }
    if (wavefront) CK(cudaMemsetAsync(ctx->wave.ray_stats, 0, 4 * sizeof(unsigned long long), ctx->stream));
    l2_window(ctx, s, true);
    CK(cudaEventRecord(ctx->ev_begin, ctx->stream));
    const bool use_graph = wavefront && !timing && (o->flags & BG_RENDER_GRAPH);
    if (total > 0 && use_graph) {
        // key: every launch parameter baked into the graph (first_sample travels in wavectl)
        bg::RenderParams rk = rp;
        rk.first_sample = 0;
        std::vector<unsigned char> key;
        auto put = [&](const void* p, size_t n) {
            const unsigned char* b = static_cast<const unsigned char*>(p);
            key.insert(key.end(), b, b + n);
        };
        put(&s->dev, sizeof(s->dev));
        put(&dc, sizeof(dc));
        put(&rk, sizeof(rk));
        put(&ctx->film, sizeof(ctx->film));
        put(&ctx->wave, sizeof(ctx->wave));
        put(&ctx->shape, sizeof(ctx->shape));
        put(&total, sizeof(total));
        if (!ctx->graph_exec || key != ctx->graph_key) {
            if (ctx->graph_exec) {
                cudaGraphExecDestroy(ctx->graph_exec);
                ctx->graph_exec = nullptr;
            }
            cudaGraph_t g = nullptr;
            CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
            int nk = bg::launch_wave_chain(s->dev, dc, rp, ctx->film, ctx->wave, total, ctx->d_err, ctx->shape,
                                           ctx->stream);
            cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
            if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaStreamEndCapture");
            ce = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
            cudaGraphDestroy(g);
            if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaGraphInstantiate");
            ctx->graph_key = key;
            ctx->graph_kernels = nk;
        }
        uint32_t ctl[4] = {0u, o->first_sample, 0u, 0u};
        CK(cudaMemcpyAsync(ctx->wave.wavectl, ctl, sizeof(ctl), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));  // ctl is a stack buffer
        CK(cudaEventRecord(ctx->ev_begin, ctx->stream));
        for (uint64_t w = 0; w < nwaves; ++w) {
            CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
            launches += (uint64_t)ctx->graph_kernels;
        }
    } else if (total > 0) {
        if (wavefront) {
            uint64_t w = 0;
            for (uint64_t item0 = 0; item0 < total; item0 += cap, ++w) {
                uint32_t nitems = (uint32_t)std::min<uint64_t>(cap, total - item0);
                launches += bg::launch_wave(s->dev, dc, rp, ctx->film, ctx->wave, item0, nitems, ctx->d_err,
                                            ctx->shape, ctx->stream,
                                            timing ? ctx->timing_ev.data() + w * ev_per_wave : nullptr);
            }
        } else if (tree) {
            const int kind = o->integrator == BG_INTEGRATOR_WHITTED ? 1
                             : (o->light_strategy == BG_LIGHT_UNIFORM_ALL ? 2 : 3);
            const bool wide = s->kind == BG_BVH_WIDE || s->kind == BG_BVH_WIDE2;
            if (o->mode == BG_MODE_PBRT && wide) {
                // breadth-first wavefront over the trees of up to W samples per wave
                const uint64_t nl = std::max<uint64_t>(s->dev.nlights, 1);
                const uint64_t per_node = kind == 1 ? nl : (kind == 2 ? 2 * nl : 2);
                const uint64_t sh_budget = 1ull << 25;  // shadow rays per level
                uint64_t W = std::min<uint64_t>({(uint64_t)kTreeWaveSamples, (uint64_t)ctx->max_queue, total,
                                                 std::max<uint64_t>(1, sh_budget / (2 * per_node))});
                W = std::max<uint64_t>(W, 1);
                const bool textured = s->dev.ntex > 0;
                if ((st = ensure_tree_wave(ctx, (uint32_t)W, (uint32_t)std::min<uint64_t>(sh_budget, 2 * W * per_node),
                                           textured)) != BG_OK)
                    return st;
                CK(cudaMemsetAsync(ctx->tree.ray_stats, 0, 2 * sizeof(unsigned long long), ctx->stream));
                uint64_t n_wave = W;
                for (uint64_t item0 = 0; item0 < total;) {
                    const uint32_t n = (uint32_t)std::min<uint64_t>(n_wave, total - item0);
                    launches += bg::launch_tree_wave(kind, s->dev, dc, rp, ctx->tree, item0, n, ctx->d_err, ctx->shape,
                                                     ctx->stream);
                    uint32_t overflow = 0;
                    CK(cudaMemcpyAsync(&overflow, ctx->tree.counters + 5, sizeof(overflow), cudaMemcpyDeviceToHost,
                                       ctx->stream));
                    CK(cudaStreamSynchronize(ctx->stream));
                    if (overflow) {  // nothing reached the film: render these samples in smaller waves
                        if (n == 1)
                            return fail(ctx, BG_ERR_UNSUPPORTED, "one sample's ray tree outgrew the tree wavefront");
                        n_wave = std::max<uint64_t>(1, n / 2);
                        continue;
                    }
                    bg::launch_tree_final(rp, ctx->film, ctx->tree, item0, n, ctx->shape, ctx->stream);
                    launches += 1;
                    item0 += n;
                }
            } else {
                const int layout = s->kind == BG_BVH_WIDE ? 8 : (s->kind == BG_BVH_WIDE2 ? 2 : 1);
                bg::launch_tree_integrator(kind, o->mode == BG_MODE_REF_COMPAT, layout, s->dev, dc, rp, ctx->film,
                                           ctx->d_err, ctx->shape, ctx->stream);
                launches += 1;
            }
        } else {
            bg::launch_megakernel(o->mode == BG_MODE_REF_COMPAT, s->dev, dc, rp, ctx->film, ctx->d_err, ctx->shape,
                                  ctx->stream);
            launches += 1;
        }
    }
    bg::launch_resolve(ctx->film, ctx->stream);
    launches += 1;
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev_end, ctx->stream));
    l2_window(ctx, s, false);
    uint32_t word = 0;
    st = check_device_error(ctx, &word);
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ctx->ev_begin, ctx->ev_end);
        stats->device_ms = ms;
        stats->samples = total;
        stats->launches = launches;
        stats->error_word = word;
        unsigned long long nan = 0;
        cudaMemcpy(&nan, ctx->film.nan_count, sizeof(nan), cudaMemcpyDeviceToHost);
        stats->nan_samples = nan;
        if (wavefront || (tree && ctx->tree.ray_stats)) {
            unsigned long long rs[2] = {0, 0};
            cudaMemcpy(rs, wavefront ? ctx->wave.ray_stats : ctx->tree.ray_stats, sizeof(rs), cudaMemcpyDeviceToHost);
            stats->extension_rays = rs[0];
            stats->shadow_rays = rs[1];
        }
        if (timing) {
            double ext = 0, shade = 0, shadow = 0;
            for (uint64_t w = 0; w < nwaves; ++w) {
                cudaEvent_t* e = ctx->timing_ev.data() + w * ev_per_wave;
                for (uint32_t b = 0; b <= o->max_depth; ++b) {
                    float a = 0, c = 0, d = 0;
                    cudaEventElapsedTime(&a, e[4 * b], e[4 * b + 1]);
                    cudaEventElapsedTime(&c, e[4 * b + 1], e[4 * b + 2]);
                    cudaEventElapsedTime(&d, e[4 * b + 2], e[4 * b + 3]);
                    ext += a;
                    shade += c;
                    shadow += d;
                }
            }
            stats->trace_ms = ext;
            stats->shade_ms = shade;
            stats->shadow_ms = shadow;
        }
    }
    if (st != BG_OK) return st;
    if (!(o->flags & BG_RENDER_NO_READBACK)) {
        CK(cudaMemcpyAsync(rgb_out, ctx->film.rgb, npix * 3 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return BG_OK;
}

bg_status bg_render_batch(bg_ctx* ctx, const bg_batch_item* items, size_t n, bg_render_stats* stats) {
    if (!ctx || !items || n == 0) return BG_ERR_INVALID;
    if (n > 65536) return fail(ctx, BG_ERR_INVALID, "at most 65536 scenes per batch");
    uint64_t total_pix = 0, total_items = 0;
    uint32_t max_depth = 0;
    uint32_t variants = 0;  // bit 0: some scene is textured, bit 1: some scene holds an infinite light
    for (size_t i = 0; i < n; ++i) {
        const bg_batch_item& it = items[i];
        bg_render_opts o = it.opts;
        o.flags = BG_RENDER_NO_READBACK;  // read-back is per item below
        bg_status st = validate_render(ctx, it.scene, &it.camera, &o, nullptr);
        if (st != BG_OK) return st;
        if (it.scene->kind != BG_BVH_WIDE)
            return fail(ctx, BG_ERR_UNSUPPORTED, "batch rendering needs scenes committed with BG_BVH_WIDE");
        if (it.opts.mode != BG_MODE_PBRT) return fail(ctx, BG_ERR_UNSUPPORTED, "batch rendering needs BG_MODE_PBRT");
        if (it.opts.integrator != BG_INTEGRATOR_PATH)
            return fail(ctx, BG_ERR_UNSUPPORTED, "batch rendering runs the path integrator only");
        if (it.scene->dev.ntex) variants |= 1u;
        if (it.scene->has_inf || it.scene->dev.sph_emis || it.scene->dev.quad_emis) variants |= 2u;
        total_pix += (uint64_t)it.camera.width * it.camera.height;
        total_items += (uint64_t)it.camera.width * it.camera.height * it.opts.spp;
        max_depth = std::max(max_depth, it.opts.max_depth);
    }
    if (total_pix >= (1ull << 31)) return fail(ctx, BG_ERR_INVALID, "batch film too large");
    CK(cudaSetDevice(ctx->device));
    bg_status st;
    if ((st = ensure_film(ctx, (uint32_t)total_pix, 1)) != BG_OK) return st;
    bg::launch_clear_film(ctx->film, ctx->stream);
    CK(cudaMemsetAsync(ctx->film.nan_count, 0, sizeof(unsigned long long), ctx->stream));
    std::vector<bg::SceneRender> tab(n);
    uint64_t pix0 = 0, item0 = 0;
    for (size_t i = 0; i < n; ++i) {
        const bg_batch_item& it = items[i];
        const uint64_t npix = (uint64_t)it.camera.width * it.camera.height;
        bg::SceneRender& r = tab[i];
        r.sc = it.scene->dev;
        r.cam = make_camera(it.camera);
        r.rp = bg::RenderParams{it.camera.width, it.camera.height, it.opts.spp, it.opts.max_depth, it.opts.first_sample,
                                it.opts.rr_threshold, it.opts.seed};
        r.rp = bg::with_camera(r.rp, r.cam, it.opts.spp);
        bg::strat_params(it.opts.sampler, it.opts.spp, it.opts.x_pixel_samples, it.opts.y_pixel_samples,
                         it.opts.sampled_dimensions, it.opts.jitter_samples, &r.rp.strat);  // validated above
        r.film = ctx->film;
        r.film.sum += 3 * pix0;
        r.film.sumsq += 3 * pix0;
        r.film.count += pix0;
        r.film.rgb += 3 * pix0;
        r.film.pass = nullptr;
        r.film.npix = (uint32_t)npix;
        r.item0 = item0;
        pix0 += npix;
        item0 += npix * it.opts.spp;
    }
    std::vector<void*> tmp;
    // the scene table lives in the context (grown when a batch needs more entries) so that the
    // captured graph below can refer to it; its contents are uploaded every call
    if (ctx->batch_tab_cap < n) {
        CK(cudaStreamSynchronize(ctx->stream));
        dfree_all(ctx, ctx->batch_allocs);
        ctx->batch_tab = nullptr;
        ctx->batch_tab_cap = 0;
        if (ctx->batch_graph) {
            cudaGraphExecDestroy(ctx->batch_graph);
            ctx->batch_graph = nullptr;
        }
        void* p;
        if ((st = dalloc(ctx, n * sizeof(bg::SceneRender), &p, &ctx->batch_allocs)) != BG_OK) return st;
        ctx->batch_tab = (bg::SceneRender*)p;
        ctx->batch_tab_cap = n;
    }
    const bg::SceneRender* d_tab = ctx->batch_tab;
    CK(cudaMemcpyAsync(ctx->batch_tab, tab.data(), n * sizeof(bg::SceneRender), cudaMemcpyHostToDevice, ctx->stream));
    const uint32_t cap = (uint32_t)std::min<uint64_t>(ctx->max_queue, std::max<uint64_t>(total_items, 1));
    if ((st = ensure_wave(ctx, cap)) != BG_OK) {
        dfree_all(ctx, tmp);
        return st;
    }
    CK(cudaMemsetAsync(ctx->wave.ray_stats, 0, 4 * sizeof(unsigned long long), ctx->stream));
    // every wave of the batch in one CUDA graph, captured once per batch shape and replayed: the
    // whole uneven batch renders with one graph launch
    std::vector<unsigned char> key;
    auto put = [&](const void* p, size_t k) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        key.insert(key.end(), b, b + k);
    };
    const uint64_t nn = n;
    put(&d_tab, sizeof(d_tab));
    put(&nn, sizeof(nn));
    put(&max_depth, sizeof(max_depth));
    put(&cap, sizeof(cap));
    put(&total_items, sizeof(total_items));
    put(&variants, sizeof(variants));
    put(&ctx->wave, sizeof(ctx->wave));
    put(&ctx->shape, sizeof(ctx->shape));
    if (!ctx->batch_graph || key != ctx->batch_key) {
        if (ctx->batch_graph) {
            cudaGraphExecDestroy(ctx->batch_graph);
            ctx->batch_graph = nullptr;
        }
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        int nk = 0;
        for (uint64_t w0 = 0; w0 < total_items; w0 += cap) {
            const uint32_t nitems = (uint32_t)std::min<uint64_t>(cap, total_items - w0);
            nk += bg::launch_wave_batch(d_tab, (uint32_t)n, max_depth, ctx->wave, w0, nitems, ctx->d_err, ctx->shape,
                                        ctx->stream, variants);
        }
        cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
        if (ce != cudaSuccess) {
            dfree_all(ctx, tmp);
            return cuda_fail(ctx, ce, "cudaStreamEndCapture (batch)");
        }
        ce = cudaGraphInstantiate(&ctx->batch_graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            ctx->batch_graph = nullptr;
            dfree_all(ctx, tmp);
            return cuda_fail(ctx, ce, "cudaGraphInstantiate (batch)");
        }
        ctx->batch_key = key;
        ctx->batch_graph_kernels = nk;
    }
    CK(cudaEventRecord(ctx->ev_begin, ctx->stream));
    uint64_t launches = (uint64_t)ctx->batch_graph_kernels;
    CK(cudaGraphLaunch(ctx->batch_graph, ctx->stream));
    bg::launch_resolve(ctx->film, ctx->stream);
    launches += 1;
    cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) {
        cudaStreamSynchronize(ctx->stream);
        dfree_all(ctx, tmp);
        return cuda_fail(ctx, le, "batch launch");
    }
    CK(cudaEventRecord(ctx->ev_end, ctx->stream));
    uint32_t word = 0;
    st = check_device_error(ctx, &word);
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ctx->ev_begin, ctx->ev_end);
        stats->device_ms = ms;
        stats->samples = total_items;
        stats->launches = launches;
        stats->error_word = word;
        unsigned long long nan = 0, rs[2] = {0, 0};
        cudaMemcpy(&nan, ctx->film.nan_count, sizeof(nan), cudaMemcpyDeviceToHost);
        cudaMemcpy(rs, ctx->wave.ray_stats, sizeof(rs), cudaMemcpyDeviceToHost);
        stats->nan_samples = nan;
        stats->extension_rays = rs[0];
        stats->shadow_rays = rs[1];
    }
    if (st == BG_OK) {
        pix0 = 0;
        for (size_t i = 0; i < n && st == BG_OK; ++i) {
            const uint64_t npix = (uint64_t)items[i].camera.width * items[i].camera.height;
            if (items[i].rgb_out) {
                cudaError_t e = cudaMemcpyAsync(items[i].rgb_out, ctx->film.rgb + 3 * pix0, npix * 3 * sizeof(float),
                                                cudaMemcpyDeviceToHost, ctx->stream);
                if (e != cudaSuccess) st = cuda_fail(ctx, e, "cudaMemcpyAsync");
            }
            pix0 += npix;
        }
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (st == BG_OK && e != cudaSuccess) st = cuda_fail(ctx, e, "cudaStreamSynchronize");
    }
    cudaStreamSynchronize(ctx->stream);
    dfree_all(ctx, tmp);
    return st;
}

bg_status bg_film_moments(bg_ctx* ctx, double* sum, double* sumsq, uint32_t* count) {
    if (!ctx) return BG_ERR_INVALID;
    if (!ctx->film.sum) return fail(ctx, BG_ERR_INVALID, "no film rendered yet");
    CK(cudaSetDevice(ctx->device));
    size_t npix = ctx->film.npix;
    if (sum) CK(cudaMemcpyAsync(sum, ctx->film.sum, npix * 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (sumsq)
        CK(cudaMemcpyAsync(sumsq, ctx->film.sumsq, npix * 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (count) CK(cudaMemcpyAsync(count, ctx->film.count, npix * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return BG_OK;
}

}  // extern "C"

// bg_internal.h - library-internal state behind the C ABI (shared by bg_api.cpp and
// bg_guide_api.cpp): the context, the scene, and the device-memory / film / wave helpers.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/bonsai_gpu.h"
#include "bg_kernels.h"

struct bg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    uint64_t cap = 0, used = 0;
    bg::ShadeFork fork{};           // streams / events of BG_TUNE_CONCURRENT_SHADE
    bg::LaunchShape shape{1, 128};
    uint32_t max_queue = 1u << 22;
    uint32_t* d_err = nullptr;
    unsigned long long* d_counters = nullptr;
    uint32_t* d_head = nullptr;
    bg::FilmBuffers film{};
    uint32_t film_w = 0, film_h = 0;
    bg::WaveBuffers wave{};
    std::vector<void*> wave_allocs;
    bg::TreeWave tree{};  // Whitted / direct-lighting wavefront (allocated on first use)
    std::vector<void*> tree_allocs;
    std::vector<void*> film_allocs;
    void* flush = nullptr;
    size_t flush_bytes = 0;
    std::vector<void*> user;
    std::unordered_map<void*, size_t> sizes;
    cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
    cudaEvent_t stage_ev[4] = {nullptr, nullptr, nullptr, nullptr};
    std::vector<cudaEvent_t> timing_ev;
    // captured wave chain (BG_RENDER_GRAPH) and the launch parameters it was captured with
    cudaGraphExec_t graph_exec = nullptr;
    std::vector<unsigned char> graph_key;
    int graph_kernels = 0;
    // batch renders: the scene table (kept, refilled per call) and the captured graph of all the
    // batch's waves, replayed while the batch's shape stays the same
    bg::SceneRender* batch_tab = nullptr;
    size_t batch_tab_cap = 0;
    std::vector<void*> batch_allocs;
    cudaGraphExec_t batch_graph = nullptr;
    std::vector<unsigned char> batch_key;
    int batch_graph_kernels = 0;
    std::unordered_set<bg_scene*> scenes;  // live scenes; orphaned (ctx = null) by bg_destroy
    std::unordered_set<bg_guide*> guides;  // live guiding networks; orphaned the same way
    size_t l2_persist_max = 0, l2_window_max = 0;  // device limits for L2 access-policy windows
    bool l2_limit_set = false;
};

struct bg_scene {
    bg_ctx* ctx = nullptr;
    std::vector<float> tri;
    std::vector<uint32_t> tri_mat;
    std::vector<int32_t> tri_light;
    // per-triangle mesh attributes (all triangles, filled with defaults for triangles without)
    std::vector<float> tri_n;         // 9 per triangle: vertex shading normals (TRI_NORMALS only)
    std::vector<float> tri_uv;        // 6 per triangle: vertex uvs
    std::vector<uint8_t> tri_flags;   // TRI_REVERSE | TRI_SWAPS | TRI_NORMALS
    bool any_normals = false, any_uvs = false, any_flags = false;
    std::vector<bg::TexInfo> tex;     // textures, level offsets into texels
    std::vector<float4> texels;
    // the infinite area light: its environment map's pyramid (in texels) and transforms
    bool has_inf = false;
    bg::TexInfo inf_map{};
    float inf_l2w[12] = {}, inf_w2l[12] = {};
    std::vector<bg_sphere> sph;
    std::vector<bg_quadric> quads;
    std::vector<bg_material> mats;
    std::vector<bg_area_light> lights;
    bool committed = false;
    uint32_t kind = BG_BVH_WIDE;
    bg::Scene dev{};
    float bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};  // bounds of all primitives
    void* hot = nullptr;   // 8-wide layout: nodes + leaf primitives, one range
    size_t hot_bytes = 0;
    std::vector<void*> allocs;
};


namespace bgi {

constexpr uint64_t kFaithfulMaxPrims = 200000;
constexpr uint32_t kTreeWaveSamples = 1u << 21;  // camera samples per Whitted / direct-lighting wave

bool triangle_light_sides(const bg_scene* s, std::vector<uint8_t>* out, std::string* why);
bg_status ensure_tree_wave(bg_ctx* ctx, uint32_t samples, uint32_t sh_cap, bool textured);
// With BG_TUNE_L2_PERSIST: marks the scene's traversal range as persisting in L2 for the launches
// that follow on the context's stream (on = false clears the window and the persisting lines).
void l2_window(bg_ctx* ctx, const bg_scene* s, bool on);
void affine_inverse(const float* xf, float* inv);

bg_status fail(bg_ctx* c, bg_status s, const std::string& msg);
bg_status cuda_fail(bg_ctx* c, cudaError_t e, const char* what);
bg_status dalloc(bg_ctx* ctx, size_t bytes, void** p, std::vector<void*>* owner);
void dfree(bg_ctx* ctx, void* p);
void dfree_all(bg_ctx* ctx, std::vector<void*>& v);
bg::Camera make_camera(const bg_camera& c);
bg_status ensure_film(bg_ctx* ctx, uint32_t w, uint32_t h);
bg_status ensure_wave(bg_ctx* ctx, uint32_t cap);
bg_status check_device_error(bg_ctx* ctx, uint32_t* word);
// Scene bounds padded slightly: p_norm = (p - lo) * inv lies in [0, 1) for every primitive.
void scene_bounds(const bg_scene* s, float lo[3], float inv[3]);
// Shared argument checks of bg_render / bg_render_guided.
bg_status validate_render(bg_ctx* ctx, const bg_scene* s, const bg_camera* cam, const bg_render_opts* o,
                          const float* rgb_out);

// Frees the device state of the context's guiding networks (bg_destroy); they keep host state only.
void guide_orphan_all(bg_ctx* ctx);

}  // namespace bgi

#define CK(call)                                                     \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) return bgi::cuda_fail(ctx, e_, #call); \
    } while (0)

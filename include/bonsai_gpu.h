/*
 * bonsai_gpu.h - C ABI of the GB300 path-tracing library (libbonsai_gpu.so).
 *
 * The library replaces the CPU render loop of the Bonsai renderer
 * (kazijawad/bonsai).  It sits exactly where the reference's
 *   trait Integrator { fn render(&self, scene: &Scene); }       src/base/integrator.rs:26-28
 *   trait SamplerIntegrator { camera(), sampler(), render(), radiance() }
 *                                                              src/base/integrator.rs:30-141
 *   PathIntegrator::new(camera, sampler, max_depth, rr_threshold)  src/integrators/path.rs:27-39
 * sit: a host integrator flattens its Scene (shapes, materials, area lights) through the
 * bg_scene_* calls once, then every bg_render call renders one film.
 *
 * Conventions (mirroring the reference's): the caller owns every host buffer; the library owns
 * all device memory; every call returns a bg_status and never aborts or throws across the ABI
 * (the reference panics instead, e.g. src/base/bsdf.rs:162).  A bg_ctx is used by one host
 * thread at a time; all work is ordered on the context's own CUDA stream.
 * Plain C types only: float xyz triplets, 32-bit ids, sizes.
 */
#ifndef BONSAI_GPU_H
#define BONSAI_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bg_status {
    BG_OK = 0,
    BG_ERR_INVALID = 1,     /* bad argument, size or scene record                     */
    BG_ERR_CUDA = 2,        /* a CUDA runtime call failed (text in bg_last_error)      */
    BG_ERR_OOM = 3,         /* device allocation failed or exceeded the memory cap     */
    BG_ERR_TIMEOUT = 4,     /* a bounded device wait ran out                           */
    BG_ERR_DEVICE = 5,      /* a device-side check raised the error word               */
    BG_ERR_UNSUPPORTED = 6, /* feature the reference has but this library does not     */
    BG_ERR_NO_DEVICE = 7    /* no CUDA device / extension built for another arch       */
} bg_status;

/* Estimator semantics.  BG_MODE_REF_COMPAT reproduces the reference PathIntegrator exactly
 * (including its defects: the path never re-spawns, src/integrators/path.rs:70-143; the MIS
 * BSDF branch follows the light direction, src/base/integrator.rs:400-431; spawn_ray caps
 * t_max at 0.9999, src/base/interaction.rs:115-121; ...).  BG_MODE_PBRT is the unbiased
 * PBRT-v3 path tracer the reference intends. */
typedef enum bg_mode { BG_MODE_REF_COMPAT = 0, BG_MODE_PBRT = 1 } bg_mode;

/* Material kinds.  MATTE = MatteMaterial with sigma 0 (src/materials/matte.rs:19-41),
 * PLASTIC = PlasticMaterial (src/materials/plastic.rs:23-53), CONDUCTOR = BSDF{
 * MicrofacetReflection(R=1, TrowbridgeReitz(a,a), FresnelConductor(1, eta, k))},
 * DIELECTRIC = BSDF{FresnelSpecular(R=1, T=1, 1.0, ior, Radiance)} with BSDF eta = ior. */
typedef enum bg_material_type {
    BG_MAT_MATTE = 0,
    BG_MAT_PLASTIC = 1,
    BG_MAT_CONDUCTOR = 2,
    BG_MAT_DIELECTRIC = 3
} bg_material_type;

typedef struct bg_material {
    uint32_t type;            /* bg_material_type                                          */
    float kd[3];              /* diffuse reflectance (matte, plastic)                      */
    float ks[3];              /* specular reflectance (plastic)                            */
    float roughness;          /* TR alpha (conductor), roughness (plastic)                 */
    uint32_t remap_roughness; /* plastic: apply TrowbridgeReitz::roughness_to_alpha        */
    float eta[3];             /* conductor eta                                             */
    float k[3];               /* conductor absorption k                                    */
    float ior;                /* dielectric index of refraction (outside medium is 1.0)    */
    float sigma;              /* matte: Oren-Nayar sigma in degrees (0 = Lambertian,
                                 src/materials/matte.rs:28-37; clamped to [0, 90])         */
    uint32_t kd_texture;      /* 0: constant kd; t > 0: texture t - 1 (matte, plastic)     */
    uint32_t ks_texture;      /* 0: constant ks; t > 0: texture t - 1 (plastic)            */
} bg_material;

/* Textures (Texture<RGBSpectrum>, src/base/texture.rs:10-12).  IMAGE = ImageTexture with its
 * MIPMap (src/textures/image.rs, src/base/mipmap.rs): `rgb` holds width*height*3 linear floats,
 * rows top to bottom (Image::pixels); width and height must be powers of two (the reference
 * resamples other sizes with the image crate's Lanczos3 filter but keeps the original
 * resolution, src/io/image.rs:28-44).  UV = UVTexture (src/textures/uv.rs): (s - floor s,
 * t - floor t, 0).  The mapping turns a shading point into (s, t) (src/base/texture.rs:22-144):
 * UV = UVMapping2D{uv_scale, uv_delta}; SPHERICAL / CYLINDRICAL = {world_to_texture} (row-major
 * 3x4 affine); PLANAR = PlanarMapping2D{vs, vt, ds, dt}. */
typedef enum bg_texture_kind { BG_TEXTURE_IMAGE = 0, BG_TEXTURE_UV = 1 } bg_texture_kind;
typedef enum bg_wrap_mode { BG_WRAP_REPEAT = 0, BG_WRAP_BLACK = 1, BG_WRAP_CLAMP = 2 } bg_wrap_mode;
typedef enum bg_mapping_kind {
    BG_MAPPING_UV = 0,
    BG_MAPPING_SPHERICAL = 1,
    BG_MAPPING_CYLINDRICAL = 2,
    BG_MAPPING_PLANAR = 3
} bg_mapping_kind;
typedef struct bg_texture {
    uint32_t kind;            /* bg_texture_kind                                           */
    uint32_t wrap;            /* bg_wrap_mode (ImageWrapMode, src/io/image.rs:11-16)       */
    uint32_t width, height;   /* image size (IMAGE)                                        */
    const float* rgb;         /* IMAGE texels; copied by bg_scene_add_texture              */
    uint32_t mapping;         /* bg_mapping_kind                                           */
    float uv_scale[2];        /* UV mapping: u_scale, v_scale                              */
    float uv_delta[2];        /* UV mapping: u_delta, v_delta                              */
    float world_to_texture[12];
    float vs[3], vt[3];       /* PLANAR mapping axes                                       */
    float ds, dt;             /* PLANAR mapping offsets                                    */
} bg_texture;

/* InfiniteAreaLight (src/lights/infinite.rs:21-79): an environment map seen from every escaping
 * ray and sampled by its luminance.  rgb: width*height*3 linear floats, rows top to bottom (row 0
 * at theta = 0), powers of two (as image textures); texels are multiplied by intensity
 * (Image::scale); light_to_world is the light's transform (row-major 3x4 affine, all zeros =
 * identity).  The scene's light list is its emitting triangles in insertion order, then the
 * infinite light. */
typedef struct bg_infinite_light {
    uint32_t width, height;
    const float* rgb;
    float intensity[3];
    float light_to_world[12];
} bg_infinite_light;

/* Triangle mesh attributes (TriangleMesh, src/shapes/triangle.rs:17-90; TriangleOptions:40-45). */
#define BG_TRI_REVERSE_ORIENTATION 1u /* TriangleOptions::reverse_orientation                   */
#define BG_TRI_SWAPS_HANDEDNESS 2u    /* the mesh transform swaps handedness (det < 0)          */

/* DiffuseAreaLight options (src/lights/diffuse.rs:26-30). */
typedef struct bg_area_light {
    float intensity[3];
    uint32_t two_sided;
} bg_area_light;

/* Sphere shape (src/shapes/sphere.rs:28-35) with a translation-only object_to_world and a full
 * z range and phi_max of 360 degrees. */
typedef struct bg_sphere {
    float center[3];
    float radius;
    uint32_t material_id;
    int32_t light_id; /* area light record (DiffuseAreaLight on the sphere) or -1 */
} bg_sphere;

/* Quadric shapes (src/shapes/{cylinder,disk,cone}.rs) with an affine object_to_world transform.
 * Both matrices are given, as the reference's Transform{m, m_inverse}: row-major 3x4 (the bottom
 * row is 0 0 0 1).  Cylinder: radius, z_min, z_max, phi_max; Disk: height, radius, inner_radius,
 * phi_max; Cone: radius, height, phi_max (degrees, clamped to [0, 360]). */
typedef enum bg_quadric_kind { BG_QUADRIC_CYLINDER = 0, BG_QUADRIC_DISK = 1, BG_QUADRIC_CONE = 2 } bg_quadric_kind;
typedef struct bg_quadric {
    uint32_t kind;
    uint32_t reverse_orientation;
    float object_to_world[12];
    float world_to_object[12];
    float radius;
    float inner_radius;
    float z_min;
    float z_max;
    float height;
    float phi_max_deg;
    uint32_t material_id;
    int32_t light_id; /* area light record or -1 (cylinders and disks; cones cannot emit) */
} bg_quadric;

/* PerspectiveCamera options (src/cameras/perspective.rs:36-46) with the camera_to_world
 * transform given as Transform::look_at(position, look_at, up) (src/base/transform.rs:152-189),
 * shutter [0,1], and film Film{full_resolution=(width,height), crop [0,1]^2, BoxFilter r=0.5,
 * scale 1, max_sample_luminance = +inf}. */
typedef struct bg_camera {
    float position[3];
    float look_at[3];
    float up[3];
    float fov_deg;
    float near_plane;
    float far_plane;
    float lens_radius;    /* thin-lens depth of field (0: pinhole), perspective.rs:127-139 */
    float focal_distance;
    uint32_t width;
    uint32_t height;
} bg_camera;

typedef struct bg_render_opts {
    uint32_t spp;          /* samples per pixel                                           */
    uint32_t max_depth;    /* PathIntegrator max_depth                                    */
    float rr_threshold;    /* PathIntegrator rr_threshold (roulette only after 3 bounces) */
    uint32_t mode;         /* bg_mode                                                     */
    uint64_t seed;         /* counter-RNG key                                             */
    uint32_t first_sample; /* index of the first sample (progressive rendering)           */
    uint32_t flags;        /* BG_RENDER_* bits                                            */
    uint32_t integrator;   /* bg_integrator (0 = PathIntegrator)                          */
    uint32_t light_strategy; /* direct lighting: bg_light_strategy                        */
    uint32_t sampler;      /* bg_sampler                                                  */
    uint32_t x_pixel_samples, y_pixel_samples; /* StratifiedSampler: spp = x * y             */
    uint32_t sampled_dimensions; /* StratifiedSampler: stratified get_1d / get_2d calls     */
    uint32_t jitter_samples;     /* StratifiedSampler: jitter inside the strata (0 / 1)     */
    uint32_t reserved;
} bg_render_opts;

/* The sampler (src/base/sampler.rs).  INDEPENDENT: every get_1d / get_2d call of a sample draws
 * from the counter-based RNG keyed by (pixel, sample, dimension).  STRATIFIED: StratifiedSampler
 * (src/samplers/stratified.rs): the first sampled_dimensions get_1d calls and get_2d calls of each
 * sample (camera film, lens and time first, then the path's calls in the reference's order) take
 * stratified values over the pixel's spp = x_pixel_samples * y_pixel_samples samples; later calls
 * draw from the counter RNG.  In REF_COMPAT mode every dimension visits the strata in the same
 * order (the reference's shuffle never swaps); in PBRT mode each dimension is permuted.  Strata are
 * defined per aligned block of spp samples (first_sample a multiple of spp starts a new block).
 * Whitted and direct lighting accept sampled_dimensions <= 1 (the camera sample's calls). */
typedef enum bg_sampler { BG_SAMPLER_INDEPENDENT = 0, BG_SAMPLER_STRATIFIED = 1 } bg_sampler;

/* The SamplerIntegrator behind bg_render.  PATH = PathIntegrator (src/integrators/path.rs);
 * WHITTED = WhittedIntegrator (src/integrators/whitted.rs): emission, every light sampled once
 * without MIS, specular reflection / transmission recursion; DIRECT = DirectLightingIntegrator
 * (src/integrators/direct.rs) with LightStrategy UniformSampleAll (every light, MIS) or
 * UniformSampleOne, and the same specular recursion.  Whitted and direct lighting evaluate the
 * BSDF without multiple lobes (the dielectric becomes SpecularReflection + SpecularTransmission
 * in PBRT mode; the reference's own materials have no specular lobes, so its recursion never
 * fires) and accept max_depth <= 30. */
typedef enum bg_integrator {
    BG_INTEGRATOR_PATH = 0,
    BG_INTEGRATOR_WHITTED = 1,
    BG_INTEGRATOR_DIRECT = 2
} bg_integrator;
typedef enum bg_light_strategy { BG_LIGHT_UNIFORM_ALL = 0, BG_LIGHT_UNIFORM_ONE = 1 } bg_light_strategy;

#define BG_RENDER_ACCUMULATE 1u  /* add to the film accumulated by earlier calls          */
#define BG_RENDER_NO_READBACK 2u /* leave the film on the device (rgb_out may be NULL)    */
#define BG_RENDER_GRAPH 4u       /* replay each sample pass from a captured CUDA graph     */
#define BG_RENDER_STAGE_TIMING 8u /* time every wavefront stage with CUDA events (stats)   */

typedef struct bg_render_stats {
    double device_ms;        /* CUDA-event time of the render on the context's stream      */
    double trace_ms;         /* time inside the closest-hit (extend) launches               */
    double shadow_ms;        /* time inside the any-hit (shadow) launches                   */
    double shade_ms;         /* time inside generate/shade/accumulate launches              */
    uint64_t samples;        /* width * height * spp                                         */
    uint64_t extension_rays; /* closest-hit queries traced                                  */
    uint64_t shadow_rays;    /* any-hit queries traced                                      */
    uint64_t launches;       /* kernels launched by this call                                */
    uint64_t nan_samples;    /* samples zeroed by the NaN / negative / inf checks            */
    uint32_t error_word;     /* device error bits (0 = none)                                 */
    uint32_t reserved;
} bg_render_stats;

/* Ray and hit records of the trace entry points (oracle a: closest-hit / any-hit parity). */
typedef struct bg_ray {
    float org[3];
    float tmax;
    float dir[3];
    float pad;
} bg_ray;

typedef struct bg_hit {
    int32_t prim; /* triangles 0..ntri-1 in insertion order, then spheres, then quadrics; -1 = miss */
    float t;
} bg_hit;

typedef struct bg_device_opts {
    int32_t device;            /* CUDA ordinal                                        */
    uint32_t max_queue_paths;  /* wavefront capacity (0 = library default)            */
    uint64_t memory_cap_bytes; /* refuse allocations beyond this total (0 = no cap)   */
    uint32_t block_size;       /* launch width for the wavefront stages (0 = default) */
    uint32_t reserved;
} bg_device_opts;

/* BVH layouts the scene builder can produce. */
typedef enum bg_bvh_kind {
    BG_BVH_WIDE = 0,           /* 8-wide compressed BVH (80 B nodes, 8-bit child boxes)      */
    BG_BVH_REFERENCE = 1,      /* binary BVH laid out and ordered as the reference's         */
    BG_BVH_REFERENCE_FIXED = 2, /* same, with the SAH bucket-index precedence bug fixed      */
    BG_BVH_WIDE2 = 3           /* 2-wide BVH, both child boxes in the parent (64 B nodes)    */
} bg_bvh_kind;

typedef struct bg_build_stats {
    double build_ms;     /* host BVH build + device upload                             */
    uint64_t nodes;      /* nodes in the layout                                        */
    uint64_t prims;      /* primitives                                                 */
    uint64_t device_bytes;
} bg_build_stats;

typedef struct bg_ctx bg_ctx;
typedef struct bg_scene bg_scene;

/* ---- context ---------------------------------------------------------------------------- */
bg_status bg_create(const bg_device_opts* opts, bg_ctx** out);
void bg_destroy(bg_ctx* ctx);
const char* bg_last_error(const bg_ctx* ctx);
const char* bg_status_string(bg_status s);
/* Overwrite a device buffer larger than L2 (used between timed passes). */
bg_status bg_flush_l2(bg_ctx* ctx);
bg_status bg_synchronize(bg_ctx* ctx);

/* ---- scene builder (replaces building BVH::new(Vec<Arc<dyn Primitive>>),
 *      src/accelerators/bvh.rs:53-89, and Scene::new, src/base/scene.rs:16-33) ------------- */
bg_status bg_scene_create(bg_ctx* ctx, bg_scene** out);
void bg_scene_destroy(bg_scene* scene);
/* Appends a material; its id is returned in *id. */
bg_status bg_scene_add_material(bg_scene* scene, const bg_material* m, uint32_t* id);
/* Appends an emission record (DiffuseAreaLight options); its id is returned in *id. */
bg_status bg_scene_add_area_light(bg_scene* scene, const bg_area_light* l, uint32_t* id);
/* Appends ntri world-space triangles (9 floats each: p0 p1 p2), one Triangle shape per entry
 * (src/shapes/triangle.rs:93-105).  light_ids may be NULL; otherwise light_ids[i] >= 0 makes
 * triangle i an emitter: one DiffuseAreaLight per triangle, as GeometricPrimitive{shape,
 * material, area_light} (src/primitives/geometric.rs:15-20). */
bg_status bg_scene_add_triangles(bg_scene* scene, const float* xyz, size_t ntri,
                                 const uint32_t* material_ids, const int32_t* light_ids);
/* As bg_scene_add_triangles with the mesh's per-vertex data: normals (9 floats per triangle:
 * world-space shading normals of p0 p1 p2, or NULL) and uvs (6 floats per triangle, or NULL for
 * the default (0,0) (1,0) (1,1)), and BG_TRI_* flags for every triangle of the call.  An emitting
 * triangle's vertex normals must all lie on one side of it (BG_ERR_UNSUPPORTED at commit). */
bg_status bg_scene_add_triangle_mesh(bg_scene* scene, const float* xyz, size_t ntri,
                                     const uint32_t* material_ids, const int32_t* light_ids,
                                     const float* normals, const float* uvs, uint32_t flags);
bg_status bg_scene_add_spheres(bg_scene* scene, const bg_sphere* spheres, size_t n);
/* Appends a texture; materials refer to it as *id + 1.  Image texels are copied and their MIPMap
 * pyramid is built here (Image::generate_pyramid, src/io/image.rs:55-114). */
bg_status bg_scene_add_texture(bg_scene* scene, const bg_texture* tex, uint32_t* id);
/* Sets the scene's InfiniteAreaLight (at most one); texels (finite, >= 0, power-of-two sizes) are
 * copied and scaled by the intensity.  Its MIPMap is built here; the 2D sampling distribution
 * (InfiniteAreaLight::new) and the search tables over its CDFs are built at commit, from the
 * committed scene's bounds (the light's world radius). */
bg_status bg_scene_add_infinite_light(bg_scene* scene, const bg_infinite_light* light);
/* Appends n cylinders / disks / cones (GeometricPrimitive{Cylinder|Disk|Cone, material}). */
bg_status bg_scene_add_quadrics(bg_scene* scene, const bg_quadric* quadrics, size_t n);
/* Builds the BVH on the host, uploads scene and BVH to the device. */
bg_status bg_scene_commit(bg_scene* scene, uint32_t bvh_kind, bg_build_stats* stats);

/* ---- launch tuning (chosen by the autotuner in bonsai_gb300/autotune.py) --------------------- */
typedef struct bg_tuning {
    uint32_t wave_paths;    /* wavefront capacity: paths per wave                                  */
    uint32_t blocks_per_sm; /* persistent grid of the wavefront stages = SMs x blocks_per_sm (x128) */
    uint32_t refill;        /* traversal: a warp fetches new rays once this many lanes are idle
                               (32 = only when the whole warp is idle)                             */
    uint32_t flags;         /* BG_TUNE_* bits                                                      */
} bg_tuning;
#define BG_TUNE_SORT_RAYS 1u /* bin each bounce's extension rays by direction octant and origin
                                cell before traversal (single-scene renders)                      */
#define BG_TUNE_L2_PERSIST 2u /* keep the 8-wide BVH (nodes + leaf primitives) resident in L2 with a
                                 persisting access-policy window during renders; the set-aside
                                 belongs to the context and ends with it.  Off by default: on the
                                 production frame it slows shading more than it helps traversal */
#define BG_TUNE_TILE_PIXELS 4u /* generate the wavefront's camera rays in 8 x 4 pixel tiles instead of
                                  scanline order (more coherent first-bounce traversal); on by
                                  default                                                        */
#define BG_TUNE_SHADOW_QUEUE_HALF 8u /* shadow-ray queue of one entry per path instead of two (saves
                                        36 B per path).  A bounce whose paths queue more shadow rays
                                        than that (each vertex may queue two: the light sample and the
                                        MIS ray toward the light) drops the excess and the render fails
                                        with BG_ERR_DEVICE (queue overflow in bg_last_error) */
#define BG_TUNE_CONCURRENT_SHADE 16u /* single-scene wavefront renders: run a bounce's material-class
                                        shade kernels side by side on the context's extra streams
                                        (joined before the shadow rays); on by default.  Films then
                                        differ from serial shading only in the order of their sums */
bg_status bg_get_tuning(const bg_ctx* ctx, bg_tuning* out);
bg_status bg_set_tuning(bg_ctx* ctx, const bg_tuning* t);

/* ---- render: replaces SamplerIntegrator::render (src/base/integrator.rs:35-133) with
 *      PathIntegrator::radiance (src/integrators/path.rs:51-146).  rgb_out is a host buffer of
 *      width*height*3 floats (row-major, y down) holding Film::write_image's pixel values
 *      (src/base/film.rs:156-202).  In REF_COMPAT mode the scene must be committed with a
 *      BG_BVH_REFERENCE* layout; PBRT mode accepts any layout. ------------------------------- */
bg_status bg_render(bg_ctx* ctx, const bg_scene* scene, const bg_camera* camera,
                    const bg_render_opts* opts, float* rgb_out, bg_render_stats* stats);
/* Per-pixel sample statistics of the film accumulated so far: sum and sum of squares of the
 * sanitized sample radiance (double, 3 per pixel each) and the sample count (u32 per pixel).
 * Any pointer may be NULL. */
bg_status bg_film_moments(bg_ctx* ctx, double* sum_rgb, double* sumsq_rgb, uint32_t* count);

/* ---- ray queries: BVH::intersect / intersect_test (src/accelerators/bvh.rs:281-423) over
 *      host arrays (copies inside the call) or device arrays (no copies). ------------------- */
bg_status bg_trace_closest(bg_ctx* ctx, const bg_scene* scene, const bg_ray* rays, size_t n,
                           bg_hit* hits);
bg_status bg_trace_any(bg_ctx* ctx, const bg_scene* scene, const bg_ray* rays, size_t n,
                       uint8_t* occluded);
bg_status bg_trace_closest_device(bg_ctx* ctx, const bg_scene* scene, const bg_ray* d_rays,
                                  size_t n, bg_hit* d_hits, float* kernel_ms);
bg_status bg_trace_any_device(bg_ctx* ctx, const bg_scene* scene, const bg_ray* d_rays,
                              size_t n, uint8_t* d_occluded, float* kernel_ms);
/* Device scratch owned by the context for the *_device calls (valid until bg_destroy). */
bg_status bg_device_alloc(bg_ctx* ctx, size_t bytes, void** d_ptr);
bg_status bg_device_free(bg_ctx* ctx, void* d_ptr);
bg_status bg_memcpy_h2d(bg_ctx* ctx, void* d_dst, const void* h_src, size_t bytes);
bg_status bg_memcpy_d2h(bg_ctx* ctx, void* h_dst, const void* d_src, size_t bytes);

/* ---- scene and film I/O ----------------------------------------------------------------------
 * OBJ::read (src/io/obj.rs:16-123): a triangle mesh from a Wavefront OBJ file, positions through
 * object_to_world (row-major 3x4, NULL = identity) and vertex normals through its inverse
 * transpose.  Triangles are the consecutive triples of all face indices in file order (as the
 * reference; polygons are not fanned); the i-th face vertex takes the i-th normal / texture index
 * of the file.  Files the reference would panic on give BG_ERR_INVALID (message in err /
 * bg_last_error).  bg_obj_read parses the positions into tri_out (9 floats per triangle, up to
 * max_tri; *ntri = all triangles); bg_obj_read_mesh also the vertex normals (9 floats per
 * triangle) and uvs (6 floats per triangle) when the file has them, and the mesh's BG_TRI_*
 * flags; bg_scene_add_obj adds the mesh, attributes included, with one material and light id. */
typedef struct bg_obj_info {
    size_t ntri;
    uint32_t has_normals;
    uint32_t has_uvs;
    uint32_t flags; /* BG_TRI_SWAPS_HANDEDNESS when the transform mirrors */
} bg_obj_info;
bg_status bg_obj_read(const char* path, const float* object_to_world, float* tri_out, size_t max_tri, size_t* ntri,
                      char* err, size_t err_len);
bg_status bg_obj_read_mesh(const char* path, const float* object_to_world, float* tri_out, float* normal_out,
                           float* uv_out, size_t max_tri, bg_obj_info* info, char* err, size_t err_len);
bg_status bg_scene_add_obj(bg_scene* scene, const char* path, const float* object_to_world, uint32_t material_id,
                           int32_t light_id, size_t* ntri);
/* Film::write_image (src/base/film.rs:156-202, src/io/image.rs:47-53), headless: an uncompressed
 * single-part scanline OpenEXR file with float B, G, R channels.  bg_write_exr writes a host RGB
 * buffer (width*height*3 floats, rows top to bottom); bg_film_write_exr the context's resolved
 * film of the last render. */
bg_status bg_write_exr(const char* path, const float* rgb, uint32_t width, uint32_t height);
bg_status bg_film_write_exr(bg_ctx* ctx, const char* path);

/* ---- uneven multi-scene batch ---------------------------------------------------------------
 * No counterpart in the reference (it renders one scene per process).  Renders every item in one
 * sequence of persistent launches: the paths of all scenes share the wavefront queues (each path
 * carries its scene index into a device table of scene, camera, render options and film slice),
 * so small and large scenes keep the GPU equally busy.  Scenes must be committed with
 * BG_BVH_WIDE and rendered in BG_MODE_PBRT with the path integrator (textures, infinite lights and
 * either sampler allowed, per item); each item's film is cleared and, when rgb_out is not
 * NULL, read back to it (width*height*3 floats).  Afterwards bg_film_moments returns the films of
 * all items concatenated in item order.  stats: device time and rays of the whole batch. */
typedef struct bg_batch_item {
    const bg_scene* scene;
    bg_camera camera;
    bg_render_opts opts; /* spp, max_depth, rr_threshold, seed, first_sample; flags unused */
    float* rgb_out;      /* host, or NULL */
} bg_batch_item;
bg_status bg_render_batch(bg_ctx* ctx, const bg_batch_item* items, size_t n, bg_render_stats* stats);

/* ---- render without device allocation ------------------------------------------------------
 * No counterpart in the reference: an addition for callers that must not allocate device memory
 * while they render, such as a plugin whose host application owns the GPU memory budget and only
 * allows allocation at load time, or a frame loop that must never block in the allocator.
 * Same semantics as bg_render, but it calls no cudaMalloc, cudaFree or other allocating routine:
 * its scratch (film moments, wavefront queues, path state, counters) lives in one static device
 * array of BG_NOALLOC_SCRATCH_BYTES bytes that every GPU loading the library holds until exit.
 * Limits: the path integrator only; at most BG_NOALLOC_MAX_PIXELS film pixels (larger films return BG_ERR_INVALID with the
 * limit in bg_last_error of the scene's context); waves of BG_NOALLOC_WAVE_PATHS paths; no
 * ACCUMULATE / STAGE_TIMING / GRAPH flags; a fixed launch shape (the context's tuned shape and
 * BG_TUNE_* settings do not apply; camera rays keep bg_render's 8 x 4 pixel-tile order).  The caller passes the committed scene, the output
 * d_rgb_out (device memory, width*height*3 floats) and a CUDA stream (NULL = default stream); the
 * call synchronizes that stream before returning.  The first call on a device resolves the
 * array's device address, so make it before any stream capture.  All calls share the array:
 * calls that overlap on the GPU race and must be serialised by the caller. */
#define BG_NOALLOC_MAX_PIXELS (512u * 512u)
#define BG_NOALLOC_WAVE_PATHS 65536u
#define BG_NOALLOC_SCRATCH_BYTES 29099008u
bg_status bg_render_noalloc(const bg_scene* scene, const bg_camera* camera, const bg_render_opts* opts,
                            float* d_rgb_out, void* cuda_stream);

/* ---- learned path guiding ------------------------------------------------------------------
 * No counterpart in the reference (its PathIntegrator samples continuation directions from the
 * BSDF only, src/integrators/path.rs:110-117).  A small network maps a shading point (position
 * normalised to the scene bounds and encoded with 12 octaves of sin/cos, shading normal,
 * outgoing direction) to two heads, each a mixture of 8 von Mises-Fisher lobes and a selection
 * probability c.  At matte, plastic and conductor vertices bg_render_guided samples with the
 * one-sample mixture c * guide + (1 - c) * BSDF of each head:
 *   head 0, the continuation: the path's next direction (path.rs:110-117) is drawn from the
 *     mixture and its throughput divided by the mixture's pdf; this head learns the radiance that
 *     arrives indirectly along a direction (what the path gathers after the next vertex);
 *   head 1, next-event estimation (estimate_direct, src/base/integrator.rs:330-437): the second
 *     strategy, which the reference draws from the BSDF to look for the chosen light, is drawn
 *     from the mixture and MIS-weighted by its pdf against the light sample; this head learns the
 *     emission a direction reaches directly, from the recorded continuations and from the light
 *     samples whose shadow rays reach the light.
 * The estimate stays unbiased whatever the network outputs.  The network (78 -> 4 x 64 ReLU ->
 * 2 x 41, BF16 weights and activations, FP32 accumulation on the tensor cores) trains online on
 * the radiance the render itself measures, with Adam.
 *
 * Parameter layout (BG_GUIDE_PARAMS floats): five layers of row-major W[out][80], biases folded
 * in as the weight of a constant-1 input column (column 78 of layer 0, column 64 of layers 1-4);
 * layers 0-3 have 64 rows (offset 5120 * l), layer 4 96 rows of which 82 are used (offset
 * 20480).  Unused rows and columns stay zero.
 * Query (BG_GUIDE_QUERY_FLOATS): p.xyz in [0,1], shading normal xyz, wo xyz.
 * Output (BG_GUIDE_OUTPUTS): head h at 41 h: lobe i: direction xyz (5i..5i+2, normalised on use),
 * log kappa (5i+3, clamped to [-2, 8]), weight logit (5i+4); selection logit at 40
 * (c = 0.95 sigmoid).
 * Training sample (BG_GUIDE_SAMPLE_FLOATS): query (9), wi xyz (3), BSDF pdf of wi, the weights
 * f |cos| L / p_proposal (luminance) of head 0 (L = indirect radiance along wi) and of head 1
 * (L = emission wi reaches), 1 unused. */
#define BG_GUIDE_PARAMS 28160u
#define BG_GUIDE_QUERY_FLOATS 9u
#define BG_GUIDE_OUTPUTS 82u
#define BG_GUIDE_SAMPLE_FLOATS 16u

typedef struct bg_guide bg_guide;

typedef struct bg_guide_opts {
    float learning_rate;       /* Adam step size (1e-3)                                        */
    float beta1, beta2, eps;   /* Adam moment decay and epsilon (0.9, 0.999, 1e-8)             */
    float alpha;               /* loss blend between the mixture and guide-only KL terms (0.5) */
    uint32_t batch_size;       /* samples per Adam step, a multiple of 128 (16384)             */
    uint32_t samples_per_pass; /* training samples gathered per 1-spp render pass (262144)     */
    uint32_t warmup_passes;    /* leading unguided passes that only gather training data (4)   */
    uint32_t flags;            /* BG_GUIDE_* bits                                               */
    uint64_t seed;             /* weight initialisation seed                                    */
    uint32_t pass_paths;       /* paths per pass: a pass renders max(1, pass_paths / pixels)
                                  spp (0 = 4194304)                                             */
    uint32_t epochs;           /* training epochs over each pass's pool (0 = 1)                 */
} bg_guide_opts;

#define BG_GUIDE_NO_FALLBACK 1u /* keep guiding even when its variance estimate is not lower  */
#define BG_GUIDE_NO_TRAIN 2u    /* render with the current weights; no online training         */
#define BG_GUIDE_NO_CONTINUATION 4u /* sample continuations from the BSDF only                */
#define BG_GUIDE_NO_NEE 8u      /* keep estimate_direct's second strategy a BSDF sample        */

typedef struct bg_guide_stats {
    uint32_t passes;         /* passes rendered by this call                                   */
    uint32_t guided_passes;  /* passes that sampled the guide mixture                          */
    uint32_t fallback;       /* 1 when plain BSDF sampling took over for the remaining passes  */
    uint32_t adam_steps;     /* optimiser steps taken by this call                             */
    double render_ms;        /* device time of the render passes                               */
    double train_ms;         /* device time of training (sample pool -> Adam)                  */
    double last_loss;        /* loss of the last training step                                 */
    double relvar_plain;     /* relative variance per sample of unguided passes (estimate)     */
    double relvar_guided;    /* the same for guided passes                                     */
    double ms_plain;         /* mean device time of an unguided pass                           */
    double ms_guided;        /* mean device time of a guided pass incl. its training           */
    uint64_t records;        /* positive-weight training records of the recording paths         */
    uint64_t pool_samples;   /* of which entered the training pool                             */
} bg_guide_stats;

/* Creates a network with seeded random weights (opts NULL = the defaults above). */
bg_status bg_guide_create(bg_ctx* ctx, const bg_guide_opts* opts, bg_guide** out);
void bg_guide_destroy(bg_guide* guide);
bg_status bg_guide_get_params(bg_guide* guide, float* params);
/* Limit, in SM clock cycles, of each tensor-core wait in the network's kernels on the guide's
 * device (every network on that device shares it); 0 restores the default of 2^31 cycles
 * (about 1 s).  A wait that runs out stops its kernel: it lets the matrix operations already
 * issued finish (under the default limit), frees its tensor memory and returns, and the call
 * that launched it returns BG_ERR_TIMEOUT; the context stays usable.  Meant for tests of that
 * path: a limit far below one operation's latency makes every launch time out. */
bg_status bg_guide_set_wait_limit(bg_guide* guide, uint64_t cycles);
/* Replaces the weights and resets the Adam state. */
bg_status bg_guide_set_params(bg_guide* guide, const float* params);
/* Network outputs for n host-side queries (out: n * BG_GUIDE_OUTPUTS floats). */
bg_status bg_guide_forward(bg_guide* guide, const float* queries, size_t n, float* out);
/* Gradient of the batch loss for n host-side samples (one batch, weights normalised by their
 * sum); grad: BG_GUIDE_PARAMS floats, loss: the batch loss.  No optimiser step. */
bg_status bg_guide_gradient(bg_guide* guide, const float* samples, size_t n, float* grad, float* loss);
/* Adam steps over n host-side samples in batches of batch_size; loss: mean batch loss. */
bg_status bg_guide_train(bg_guide* guide, const float* samples, size_t n, float* loss);
/* Copies the training pool gathered by the last bg_render_guided pass to the host: at most max_n
 * samples of BG_GUIDE_SAMPLE_FLOATS floats; *n_out = samples copied. */
bg_status bg_guide_pool(bg_guide* guide, float* out, size_t max_n, size_t* n_out);
/* Device timing of the network kernels (CUDA events on the context's stream, after one untimed
 * run of each): `reps` training steps on the first batch_size of n host samples (forward +
 * backward + Adam; the weights change) and `reps` inference passes over nq host queries (the
 * parsed-mixture output the renderer uses).  Outputs: mean ms per training step and per
 * inference pass. */
bg_status bg_guide_time(bg_guide* guide, const float* samples, size_t n, const float* queries, size_t nq,
                        uint32_t reps, double* train_step_ms, double* infer_ms);
/* Device evaluation of one head's mixture for given raw outputs (test entry): per item raw (41), u (3),
 * w (3), p_bsdf (1) -> out (48): sampled direction xyz, pdf of it, pdf of w, c, loss and its
 * gradient (out[7] = d/d raw[40], out[8..47] = d/d raw[0..39]) for a unit-weight sample at w. */
bg_status bg_guide_mixture_eval(bg_guide* guide, const float* raw, const float* u, const float* w,
                                const float* p_bsdf, size_t n, float* out);
/* Progressive guided render of opts->spp samples per pixel in passes of max(1, pass_paths / pixels)
 * spp (PBRT mode, wide BVH layouts; the last pass may be shorter).  The first
 * warmup_passes passes rendered with this network sample the BSDF and gather training data; later
 * passes sample the guide mixture and keep training after every pass.  Unless
 * BG_GUIDE_NO_FALLBACK is set, guiding stops for good (plain BSDF sampling, no training) once
 * its relative variance per sample times pass time, averaged over the last 32 guided passes
 * (checked from the 64th guided pass on), is not lower than that of the unguided passes.  Warm-up count, fallback and the variance
 * estimates persist in the guide across calls, so a long render can be issued in chunks (with
 * BG_RENDER_ACCUMULATE and increasing first_sample).  Film, flags and rgb_out as in bg_render;
 * guide_stats counts this call's passes and reports the running estimates.  The path integrator
 * only (BG_ERR_UNSUPPORTED otherwise); textured scenes, infinite lights and the stratified sampler
 * (strata follow the global sample index, so passes keep them) are supported. */
bg_status bg_render_guided(bg_ctx* ctx, const bg_scene* scene, bg_guide* guide, const bg_camera* camera,
                           const bg_render_opts* opts, float* rgb_out, bg_render_stats* stats,
                           bg_guide_stats* guide_stats);

#ifdef __cplusplus
}
#endif

#endif /* BONSAI_GPU_H */

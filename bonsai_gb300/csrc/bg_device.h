// bg_device.h - device-resident scene layout shared by the host driver and the kernels.
//
// HBM layout (all arrays 16-byte aligned, read with 128-bit loads):
//   tri[3*i+k]   float4 : triangle i vertex k in insertion order; w of k=0 = material id,
//                         w of k=1 = emission record (int, -1 none), w of k=2 = light index or -1
//   sph[i]       float4 : sphere center.xyz, radius; sph_mat[i] material id
//   mats[m]      Material : constant-texture parameters, alpha already remapped/clamped
//   ref_nodes    RefNode  : binary BVH in the reference's flattened DFS order (32 B/node)
//   ref_order    uint32   : ordered_primitives of the reference build (prim ids)
//   nodes        Bvh2Node : 2-wide BVH, both children's boxes in the parent (64 B/node)
//   leaf_prims   float4x3 : primitives in leaf order (48 B each; triangle p0 p1 p2, or sphere
//                           center/radius); w of the first float4 = prim id (bit 31: sphere)
//   tri_flags    uint8    : per triangle TRI_* bits (null when no triangle has attributes)
//   tri_ns[3*i+k] float4  : shading normal of triangle i vertex k (TRI_NORMALS triangles only)
//   tri_uv[3*i+k] float2  : uv of triangle i vertex k (null: the default (0,0) (1,0) (1,1))
//   tex[t]       TexInfo  : image / uv texture t with its mapping and MIPMap level table
//   texels       float4   : every texture level, rows top to bottom, rgb + 0
#pragma once
#include <cstdint>

#ifndef __CUDACC__
#include <vector_types.h>
#endif

namespace bg {

struct Material {
    uint32_t type;  // bg_material_type
    float kd[3];
    float ks[3];
    float alpha;    // TR alpha: max(roughness or roughness_to_alpha(roughness), 0.001)
    float eta[3];
    float k[3];
    float ior;
    uint32_t kd_tex;  // 0: constant kd, t: texture t - 1 (matte, plastic)
    float sigma;      // matte: Oren-Nayar sigma in degrees, clamped to [0, 90] (0: Lambertian)
    float on_a, on_b; // Oren-Nayar A and B of OrenNayer::new (src/bxdfs/oren_nayer.rs:20-30)
    uint32_t ks_tex;  // 0: constant ks, t: texture t - 1 (plastic)
    uint32_t pad;
};

// Triangle attribute bits: TriangleOptions::reverse_orientation, Transform::swaps_handedness of
// the mesh transform, and per-vertex shading normals (TriangleMesh::normal, triangle.rs:17-90).
// LFLIP / SFLIP (computed when the scene is committed): the surface normal of a hit
// (triangle.rs:299-307 and Interaction::set_shading_geometry) / of a sampled point
// (triangle.rs:534-545) is -normalize(cross(p0 - p2, p1 - p2)).  Both depend only on the
// triangle as long as its vertex normals lie on one side of it, which the host checks for
// emitting triangles; next-event estimation reads these bits instead of the vertex normals.
enum : uint8_t { TRI_REVERSE = 1, TRI_SWAPS = 2, TRI_NORMALS = 4, TRI_LFLIP = 8, TRI_SFLIP = 16 };

// ImageTexture / UVTexture with their TextureMapping2D (src/textures/{image,uv}.rs,
// src/base/texture.rs) and the MIPMap pyramid (src/base/mipmap.rs, src/io/image.rs:55-114).
enum : uint32_t { TEX_IMAGE = 0, TEX_UV = 1 };
enum : uint32_t { WRAP_REPEAT = 0, WRAP_BLACK = 1, WRAP_CLAMP = 2 };
enum : uint32_t { MAP_UV = 0, MAP_SPHERICAL = 1, MAP_CYLINDRICAL = 2, MAP_PLANAR = 3 };
constexpr int TEX_MAX_LEVELS = 16;
struct TexInfo {
    uint32_t kind, wrap, mapping, nlevels;
    float su, sv, du, dv;  // UVMapping2D scales and deltas
    float m[3][4];         // world_to_texture (spherical / cylindrical), affine rows
    float vs[3], ds;       // PlanarMapping2D
    float vt[3], dt;
    uint32_t lw[TEX_MAX_LEVELS], lh[TEX_MAX_LEVELS];
    uint32_t loff[TEX_MAX_LEVELS];  // first texel of each level in `texels`
};

struct Emission {
    float intensity[3];
    uint32_t two_sided;
};

struct RefNode {   // BVHNode (src/accelerators/bvh.rs:25-31), flattened like BVH::flatten
    float mn[3];
    float mx[3];
    uint32_t offset;      // primitive_offset (leaf) or second_child_offset (interior)
    uint32_t count_axis;  // (count << 2) | axis; count 0 = interior
};

struct Bvh2Node {
    float4 c0xy;   // child0 lo.x hi.x lo.y hi.y
    float4 c1xy;   // child1 lo.x hi.x lo.y hi.y
    float4 c01z;   // child0 lo.z hi.z, child1 lo.z hi.z
    int4 child;    // x,y: >=0 inner node; <0: ~first leaf prim; z,w: leaf prim counts
};

// 8-wide compressed node (after Ylitie, Karras, Laine, HPG 2017): 80 B, read as five 128-bit loads.
// Child boxes are 8-bit offsets on a per-node grid: lo = p + 2^(e-127) * qlo, hi = p + 2^(e-127) * qhi.
// Slot s holds an internal child (bit s of imask), a leaf of one or two primitives (bit s of
// leafmask; of twomask when two) or nothing (the inverted box qlo = 255, qhi = 0, which no ray
// enters).  Internal children are stored contiguously from child_base, leaf primitives from
// tri_base, both in slot order; slots are assigned so that a ray in direction octant o reaches
// slot o's child first.
struct Bvh8Node {
    float p[3];
    uint8_t e[3];
    uint8_t imask;
    uint32_t child_base;
    uint32_t tri_base;
    uint8_t leafmask, twomask, pad[6];
    uint8_t qlo_x[8], qlo_y[8], qlo_z[8];
    uint8_t qhi_x[8], qhi_y[8], qhi_z[8];
};
static_assert(sizeof(Bvh8Node) == 80, "Bvh8Node must be 80 bytes");

// InfiniteAreaLight (src/lights/infinite.rs): the environment map's MIPMap (a TexInfo over the
// shared texel array, repeat wrap), its transforms, the scene's bounding sphere and the
// Distribution2D over a (2w x 2h) luminance * sin(theta) image (src/base/sampling.rs:10-118):
// row v's conditional cdf at cond_cdf[v * (nu + 1)], its function values at cond_func[v * nu],
// its integral in cond_int[v]; the marginal over rows in marg_cdf / marg_func / marg_int.
struct InfLight {
    TexInfo map;
    float l2w[3][4], w2l[3][4];
    float center[3], radius;
    uint32_t nu, nv;
    const float* cond_cdf;
    const float* cond_func;
    const float* cond_int;
    const float* marg_cdf;
    const float* marg_func;
    float marg_int;
    // Guide tables (power-of-two bucket counts gu, gv): entry k of a CDF's table is its
    // find_interval at u = k / g, so a search for u starts within [table[k], table[k + 1]],
    // k = floor(u * g).  Row v's conditional table at cond_guide[v * (gu + 1)].
    uint32_t gu, gv;
    const uint32_t* cond_guide;
    const uint32_t* marg_guide;
};
// Light-list entry of the infinite light in Scene::light_prims (area lights hold their triangle).
constexpr uint32_t LIGHT_INFINITE = 0xFFFFFFFFu;

// StratifiedSampler options of a render (src/samplers/stratified.rs:32-37).
struct StratParams {
    uint32_t dims;    // sampled_dimensions (0: every call draws from the counter RNG)
    uint32_t nx, ny;  // x_pixel_samples, y_pixel_samples
    uint32_t jitter;  // jitter_samples
};

struct Camera {   // PerspectiveCamera (src/cameras/perspective.rs:117-175)
    float r2c[4][4];  // raster_to_camera.m
    float c2w[4][4];  // camera_to_world.m
    uint32_t width, height;
    float dxc[3], dyc[3];  // dx_camera, dy_camera: raster one-pixel steps in camera space
    float lens_radius, focal_distance;  // thin lens (lens_radius 0: pinhole)
};

// Quadric record (8 x float4 = 128 B): rows 0-2 object_to_world (3x4), rows 3-5 world_to_object,
// row 6 = radius, inner_radius, z_min, z_max; row 7 = height, phi_max (radians),
// flags (kind | reverse << 8 | swaps_handedness << 9) as bits, material id as bits.
constexpr int QUADRIC_F4 = 8;

struct Scene {
    const float4* tri;
    uint32_t ntri;
    uint32_t nsph;
    const float4* quads;  // QUADRIC_F4 per quadric
    uint32_t nquad;
    uint32_t pad2;
    const float4* sph;
    const uint32_t* sph_mat;
    const int32_t* sph_emis;   // emission record per sphere (-1 none); null: no emitting sphere
    const int32_t* quad_emis;  // the same per quadric
    const Material* mats;
    const Emission* emis;
    const uint32_t* light_prims;  // Scene::lights order: one DiffuseAreaLight per emitting triangle
    uint32_t nlights;
    uint32_t pad0;
    const RefNode* ref_nodes;
    const uint32_t* ref_order;
    uint32_t ref_nnodes;
    uint32_t n_nodes;
    const Bvh2Node* nodes;
    const float4* leaf_prims;   // leaf order of whichever wide layout is built
    const Bvh8Node* nodes8;
    uint32_t n_nodes8;
    uint32_t ntex;
    const uint8_t* tri_flags;
    const float4* tri_ns;
    const float2* tri_uv;
    const TexInfo* tex;
    const float4* texels;
    const InfLight* inf;  // the infinite light, or null
    const uint8_t* prim_cls;  // material class (bg_material_type) per primitive: 1 B, stays in L2
};

enum : uint32_t {
    ERR_STACK_OVERFLOW = 1u,
    ERR_QUEUE_OVERFLOW = 2u,
    ERR_BAD_PRIM = 4u,
    ERR_BAD_NODE = 8u,
    ERR_GUIDE_TIMEOUT = 16u,  // a tensor-core wait of the guiding network gave up
};

constexpr uint32_t SPHERE_BIT = 0x80000000u;
constexpr uint32_t QUADRIC_BIT = 0x40000000u;
constexpr int TRAVERSAL_STACK = 64;

}  // namespace bg

// bg_bvh.h - host BVH builders.
#pragma once
#include <cstdint>
#include <vector>

#include "../../include/bonsai_gpu.h"
#include "bg_device.h"

namespace bg {

struct HostPrims {
    const float* tri;        // 9 floats per triangle
    uint32_t ntri;
    const bg_sphere* sph;
    uint32_t nsph;
    const bg_quadric* quad = nullptr;
    uint32_t nquad = 0;
    uint32_t count() const { return ntri + nsph + nquad; }
};

// World-space bounds of primitive i (the boxes the builders use).
void prim_bounds(const HostPrims& p, uint32_t i, float lo[3], float hi[3]);

// BVH::new (src/accelerators/bvh.rs:53-269): 16-bucket SAH, leaves of up to 256 primitives,
// DFS-preorder flattening.  faithful = true keeps the bucket index `16 * (offset as usize)`
// (bvh.rs:154-155, which only ever yields buckets 0 and 15); false uses floor(16 * offset).
struct RefBvh {
    std::vector<RefNode> nodes;
    std::vector<uint32_t> order;
};
bool build_reference_bvh(const HostPrims& p, bool faithful, RefBvh* out, uint64_t max_prims_faithful);

// The library's own 2-wide BVH: binned SAH (32 bins per axis), up to 8 primitives per leaf,
// children ordered for a depth-first layout; leaf primitives copied in leaf order.
struct Bvh2 {
    std::vector<Bvh2Node> nodes;
    std::vector<float4> leaf_prims;  // 3 per primitive
};
void build_bvh2(const HostPrims& p, Bvh2* out, int threads);

// 8-wide compressed BVH: binary SAH BVH with leaves of at most 2 primitives, collapsed greedily
// (the largest-area internal child is opened until 8 children, then leaves of two primitives are
// split while slots are free), child slots assigned by octant, boxes quantised to 8 bits
// (conservative floor / ceil).
struct Bvh8 {
    std::vector<Bvh8Node> nodes;
    std::vector<float4> leaf_prims;  // 3 per primitive, node-contiguous
};
void build_bvh8(const HostPrims& p, Bvh8* out);

}  // namespace bg

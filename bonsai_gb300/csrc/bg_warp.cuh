// bg_warp.cuh - warp-level queue helpers shared by the wavefront translation units.
#pragma once
#include "bg_shapes.cuh"

namespace bg {

constexpr unsigned FULL = 0xffffffffu;

BG_D uint32_t lane_id() { return threadIdx.x & 31u; }

BG_D uint32_t warp_fetch(uint32_t* head) {
    uint32_t base = 0;
    if (lane_id() == 0) base = atomicAdd(head, 32u);
    return __shfl_sync(FULL, base, 0);
}
// Warp-aggregated append: every lane of the warp must call it; returns the slot of lanes with pred.
BG_D uint32_t warp_append(uint32_t* counter, bool pred) {
    uint32_t mask = __ballot_sync(FULL, pred);
    if (mask == 0) return 0;
    uint32_t leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane_id() == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(FULL, base, leader);
    return base + (uint32_t)__popc(mask & ((1u << lane_id()) - 1u));
}

BG_D Ray load_ray(float4 o, float4 d) {
    Ray r;
    r.o = f4xyz(o);
    r.t_max = o.w;
    r.d = f4xyz(d);
    r.time = d.w;
    return r;
}

}  // namespace bg

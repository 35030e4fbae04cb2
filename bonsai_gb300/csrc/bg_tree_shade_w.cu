// bg_tree_shade_w.cu - the tree wavefront's shade kernel for the Whitted integrator.
#include "bg_tree_wave.cuh"

namespace bg {

void launch_tw_shade_whitted(const Scene& sc, const RenderParams& rp, const TreeWave& tw, uint32_t d, uint64_t item0,
                             uint32_t* err, dim3 grid, dim3 block, cudaStream_t s) {
    if (tw.textured) k_tw_shade<true, 1><<<grid, block, 0, s>>>(sc, rp, tw, d, item0, err);
    else k_tw_shade<false, 1><<<grid, block, 0, s>>>(sc, rp, tw, d, item0, err);
}

}  // namespace bg

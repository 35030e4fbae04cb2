// bg_tree_shade_d.cu - the tree wavefront's shade kernels for the direct-lighting integrator
// (kind 2: UniformSampleAll, 3: UniformSampleOne).
#include "bg_tree_wave.cuh"

namespace bg {

void launch_tw_shade_direct(int kind, const Scene& sc, const RenderParams& rp, const TreeWave& tw, uint32_t d,
                            uint64_t item0, uint32_t* err, dim3 grid, dim3 block, cudaStream_t s) {
    if (kind == 2) {
        if (tw.textured) k_tw_shade<true, 2><<<grid, block, 0, s>>>(sc, rp, tw, d, item0, err);
        else k_tw_shade<false, 2><<<grid, block, 0, s>>>(sc, rp, tw, d, item0, err);
    } else {
        if (tw.textured) k_tw_shade<true, 3><<<grid, block, 0, s>>>(sc, rp, tw, d, item0, err);
        else k_tw_shade<false, 3><<<grid, block, 0, s>>>(sc, rp, tw, d, item0, err);
    }
}

}  // namespace bg

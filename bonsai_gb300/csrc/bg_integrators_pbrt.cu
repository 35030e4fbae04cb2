// bg_integrators_pbrt.cu - the one-thread-per-sample Whitted and direct-lighting kernel in PBRT mode
// over the reference layout.
#include "bg_tree.cuh"

namespace bg {

void launch_tree_pbrt(int kind, const Scene& sc, const Camera& cam, const RenderParams& rp, const FilmBuffers& film,
                      uint32_t* err, dim3 grid, dim3 block, cudaStream_t s) {
    k_tree<false, 1><<<grid, block, 0, s>>>(sc, cam, rp, film, kind, err);
}

}  // namespace bg

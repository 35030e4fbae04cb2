// bg_integrators.cu - the Whitted and direct-lighting integrators one thread per sample
// (bg_tree.cuh) over the reference layout: the REF_COMPAT launch here, the PBRT launch in
// bg_integrators_pbrt.cu.  PBRT renders on the wide layouts take the breadth-first tree wavefront
// (bg_tree_wave.cu) instead.
#include "bg_tree.cuh"

namespace bg {

// The host routes REF_COMPAT and reference-layout renders here (both run on the reference layout).
void launch_tree_integrator(int kind, bool ref_compat, int layout, const Scene& sc, const Camera& cam,
                            const RenderParams& rp, const FilmBuffers& film, uint32_t* err, const LaunchShape& ls,
                            cudaStream_t s) {
    (void)layout;  // always 1
    dim3 grid(ls.sms * 8), block(128);
    if (ref_compat) k_tree<true, 1><<<grid, block, 0, s>>>(sc, cam, rp, film, kind, err);
    else launch_tree_pbrt(kind, sc, cam, rp, film, err, grid, block, s);
}

}  // namespace bg

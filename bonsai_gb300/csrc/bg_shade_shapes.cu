// bg_shade_shapes.cu - single-scene shade launches for scenes whose light list holds emitting
// spheres or quadrics (and possibly the infinite light): variants with the general light code,
// textures resolved per scene at run time.
#include "bg_wave.cuh"

namespace bg {

int launch_shade_shapes(const Scene& sc, const RenderParams& rp, const FilmBuffers& film, const WaveBuffers& wb,
                        uint32_t b, uint32_t* err, dim3 grid, dim3 block, cudaStream_t s) {
    const GuideWave gw{};
    k_shade<CLS_MISS><<<grid, block, 0, s>>>(sc, rp, film, wb, gw, b, err, nullptr);
    k_shade<0, false, false, true, true, true><<<grid, block, 0, s>>>(sc, rp, film, wb, gw, b, err, nullptr);
    k_shade<1, false, false, true, true, true><<<grid, block, 0, s>>>(sc, rp, film, wb, gw, b, err, nullptr);
    k_shade<2, false, false, false, true, true><<<grid, block, 0, s>>>(sc, rp, film, wb, gw, b, err, nullptr);
    k_shade<3, false, false, false, true, true><<<grid, block, 0, s>>>(sc, rp, film, wb, gw, b, err, nullptr);
    return 5;
}

}  // namespace bg

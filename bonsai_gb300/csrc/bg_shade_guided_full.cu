// bg_shade_guided_full.cu - the guided render's shade launches for scenes with
// textures or an infinite light: variants that filter textures (matte, plastic) and sample the
// infinite light, both resolved per scene at run time.
#include "bg_wave.cuh"

namespace bg {

int launch_shade_guided_full(const Scene& sc, const RenderParams& rp, const FilmBuffers& film, const WaveBuffers& wb,
                             const GuideWave& gw, uint32_t b, uint32_t* err, dim3 grid, dim3 block,
                             cudaStream_t s, const ShadeFork* fork) {
    const ClassStreams cs = shade_fork(s, fork);
    const cudaStream_t* st = cs.st;
    k_shade<0, false, true, true, true><<<grid, block, 0, st[0]>>>(sc, rp, film, wb, gw, b, err, nullptr);
    k_shade<1, false, true, true, true><<<grid, block, 0, st[1]>>>(sc, rp, film, wb, gw, b, err, nullptr);
    k_shade<2, false, true, false, true><<<grid, block, 0, st[2]>>>(sc, rp, film, wb, gw, b, err, nullptr);
    k_shade<3, false, true, false, true><<<grid, block, 0, st[3]>>>(sc, rp, film, wb, gw, b, err, nullptr);
    k_shade<CLS_MISS, false, true><<<grid, block, 0, st[CLS_MISS]>>>(sc, rp, film, wb, gw, b, err, nullptr);
    shade_join(s, fork);
    return 5;
}

}  // namespace bg

// bg_shade_aux.cu - the shade launches of guided renders (training records, network mixtures) and
// of batch renders (per-path scenes).
#include "bg_wave.cuh"

namespace bg {

int launch_shade_guided(const Scene& sc, const RenderParams& rp, const FilmBuffers& film, const WaveBuffers& wb,
                        const GuideWave& gw, uint32_t b, uint32_t* err, dim3 grid, dim3 block, cudaStream_t s,
                        const ShadeFork* fork) {
    if (sc.ntex || general_lights(sc))
        return launch_shade_guided_full(sc, rp, film, wb, gw, b, err, grid, block, s, fork);
    const ClassStreams cs = shade_fork(s, fork);
    const cudaStream_t* st = cs.st;
    k_shade<0, false, true><<<grid, block, 0, st[0]>>>(sc, rp, film, wb, gw, b, err, nullptr);
    k_shade<1, false, true><<<grid, block, 0, st[1]>>>(sc, rp, film, wb, gw, b, err, nullptr);
    k_shade<2, false, true><<<grid, block, 0, st[2]>>>(sc, rp, film, wb, gw, b, err, nullptr);
    k_shade<3, false, true><<<grid, block, 0, st[3]>>>(sc, rp, film, wb, gw, b, err, nullptr);
    k_shade<CLS_MISS, false, true><<<grid, block, 0, st[CLS_MISS]>>>(sc, rp, film, wb, gw, b, err, nullptr);
    shade_join(s, fork);
    return 5;
}

int launch_shade_batch(const SceneRender* tab, const WaveBuffers& wb, uint32_t b, uint32_t* err, dim3 grid, dim3 block,
                       cudaStream_t s, bool full) {
    const Scene sc{};
    const RenderParams rp{};
    const FilmBuffers film{};
    const GuideWave gw{};
    k_shade<CLS_MISS, true><<<grid, block, 0, s>>>(sc, rp, film, wb, gw, b, err, tab);
    if (full) {  // textures (matte, plastic) and the infinite light's next-event estimation, per scene
        k_shade<0, true, false, true, true><<<grid, block, 0, s>>>(sc, rp, film, wb, gw, b, err, tab);
        k_shade<1, true, false, true, true><<<grid, block, 0, s>>>(sc, rp, film, wb, gw, b, err, tab);
        k_shade<2, true, false, false, true><<<grid, block, 0, s>>>(sc, rp, film, wb, gw, b, err, tab);
        k_shade<3, true, false, false, true><<<grid, block, 0, s>>>(sc, rp, film, wb, gw, b, err, tab);
    } else {
        k_shade<0, true><<<grid, block, 0, s>>>(sc, rp, film, wb, gw, b, err, tab);
        k_shade<1, true><<<grid, block, 0, s>>>(sc, rp, film, wb, gw, b, err, tab);
        k_shade<2, true><<<grid, block, 0, s>>>(sc, rp, film, wb, gw, b, err, tab);
        k_shade<3, true><<<grid, block, 0, s>>>(sc, rp, film, wb, gw, b, err, tab);
    }
    return 5;
}

}  // namespace bg

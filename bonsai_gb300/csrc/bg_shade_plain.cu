// bg_shade_plain.cu - the shade launches of single-scene wavefront renders: one kernel per
// material class (misses included), in the variants for textured scenes and for scenes whose
// light list holds the infinite light.
#include "bg_wave.cuh"

namespace bg {

int launch_shade_plain(const Scene& sc, const RenderParams& rp, const FilmBuffers& film, const WaveBuffers& wb,
                       uint32_t b, uint32_t* err, dim3 grid, dim3 block, cudaStream_t s, const ShadeFork* fork) {
    const GuideWave gw{};
    if (sc.sph_emis || sc.quad_emis) return launch_shade_shapes(sc, rp, film, wb, b, err, grid, block, s);
    const ClassStreams cs = shade_fork(s, fork);
    const cudaStream_t* st = cs.st;
    if (sc.inf) {  // the light list holds the infinite light
        if (sc.ntex) {
            k_shade<0, false, false, true, true, false><<<grid, block, 0, st[0]>>>(sc, rp, film, wb, gw, b, err, nullptr);
            k_shade<1, false, false, true, true, false><<<grid, block, 0, st[1]>>>(sc, rp, film, wb, gw, b, err, nullptr);
        } else {
            k_shade<0, false, false, false, true, false><<<grid, block, 0, st[0]>>>(sc, rp, film, wb, gw, b, err, nullptr);
            k_shade<1, false, false, false, true, false><<<grid, block, 0, st[1]>>>(sc, rp, film, wb, gw, b, err, nullptr);
        }
        k_shade<2, false, false, false, true, false><<<grid, block, 0, st[2]>>>(sc, rp, film, wb, gw, b, err, nullptr);
        k_shade<3, false, false, false, true, false><<<grid, block, 0, st[3]>>>(sc, rp, film, wb, gw, b, err, nullptr);
    } else if (sc.ntex) {
        k_shade<0, false, false, true><<<grid, block, 0, st[0]>>>(sc, rp, film, wb, gw, b, err, nullptr);
        k_shade<1, false, false, true><<<grid, block, 0, st[1]>>>(sc, rp, film, wb, gw, b, err, nullptr);
        k_shade<2><<<grid, block, 0, st[2]>>>(sc, rp, film, wb, gw, b, err, nullptr);
        k_shade<3><<<grid, block, 0, st[3]>>>(sc, rp, film, wb, gw, b, err, nullptr);
    } else {
        k_shade<0><<<grid, block, 0, st[0]>>>(sc, rp, film, wb, gw, b, err, nullptr);
        k_shade<1><<<grid, block, 0, st[1]>>>(sc, rp, film, wb, gw, b, err, nullptr);
        k_shade<2><<<grid, block, 0, st[2]>>>(sc, rp, film, wb, gw, b, err, nullptr);
        k_shade<3><<<grid, block, 0, st[3]>>>(sc, rp, film, wb, gw, b, err, nullptr);
    }
    // escaped rays
    k_shade<CLS_MISS><<<grid, block, 0, st[CLS_MISS]>>>(sc, rp, film, wb, gw, b, err, nullptr);
    shade_join(s, fork);
    return 5;
}

}  // namespace bg

// bg_film.cuh - film accumulation on the device (shared by the path wavefront, the megakernels and
// the Whitted / direct-lighting integrators).
#pragma once
#include "bg_kernels.h"
#include "bg_math.cuh"

namespace bg {

// FilmTile::add_sample with the box filter (r = 0.5: weight 1 to the sample's own pixel) after
// the radiance sanity checks of SamplerIntegrator::render (src/base/integrator.rs:91-120).
BG_D void film_add(const FilmBuffers& f, uint32_t pix, RGB L) {
    float y = luminance(L);
    if (is_nan(L) || y < -1e-5f || isinf(y)) {
        L = rgb(0.0f);
        atomicAdd(f.nan_count, 1ull);
    }
    double r = L.r, g = L.g, b = L.b;
    atomicAdd(&f.sum[3 * pix + 0], r);
    atomicAdd(&f.sum[3 * pix + 1], g);
    atomicAdd(&f.sum[3 * pix + 2], b);
    atomicAdd(&f.sumsq[3 * pix + 0], r * r);
    atomicAdd(&f.sumsq[3 * pix + 1], g * g);
    atomicAdd(&f.sumsq[3 * pix + 2], b * b);
    atomicAdd(&f.count[pix], 1u);
    if (f.pass) {
        atomicAdd(&f.pass[3 * pix + 0], L.r);
        atomicAdd(&f.pass[3 * pix + 1], L.g);
        atomicAdd(&f.pass[3 * pix + 2], L.b);
    }
}

}  // namespace bg

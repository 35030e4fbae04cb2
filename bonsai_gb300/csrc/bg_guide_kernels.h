// bg_guide_kernels.h - launch interface of the guiding-network kernels (bg_guide.cu).
#pragma once
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "bg_kernels.h"

namespace bg {

struct GuideTrainArgs {
    const uint8_t* wpack;    // BF16 weight image
    const float4* samples;   // 4 float4 per sample
    uint32_t n;              // samples (rows past n are zero-weight)
    const float* wsum;       // sum of the batch's weights (device scalar)
    float alpha;             // loss blend, see guide_loss_grad
    float* grad;             // FP32 gradient accumulator (GUIDE_PARAMS)
    float* stats;            // [0] += loss, [1] += samples with weight > 0
    uint32_t* step;          // Adam step counter, incremented once per launch (null: gradient only)
    uint32_t* err;           // error word
};

struct GuideAdam {
    float lr, beta1, beta2, eps;
};

void launch_guide_infer(const uint8_t* wpack, const float4* query, const uint32_t* count, uint32_t max_n, float* raw,
                        uint32_t* err, int sms, cudaStream_t s);
void launch_guide_train(const GuideTrainArgs& a, cudaStream_t s);
void launch_guide_adam(float* p, float* m, float* v, float* g, uint8_t* wpack, const uint32_t* step,
                       const GuideAdam& h, cudaStream_t s);
void launch_guide_pack(const float* p, uint8_t* wpack, cudaStream_t s);
void launch_guide_wsum(const float4* samples, uint32_t n, uint32_t batch, float* wsum, cudaStream_t s);
// Relative variance of this pass's samples (film.pass) against the mean of the earlier passes:
// out[0] += sum over pixels with >= 2 samples and channels of (x - m)^2 / (m^2 + 0.01) * (n - 1) / n,
// out[1] += number of terms.  (n - 1) / n removes the variance of m itself, so out[0] / out[1]
// estimates the relative variance of one sample.
void launch_pass_relvar(const FilmBuffers& film, double* out, cudaStream_t s);
void launch_guide_mixture_eval(const float* raw, const float* u, const float* w, const float* pb, uint32_t n,
                               float alpha, float* out, cudaStream_t s);

}  // namespace bg

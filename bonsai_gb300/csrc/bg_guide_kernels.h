// bg_guide_kernels.h - launch interface of the guiding-network kernels (bg_guide.cu).
#pragma once
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "bg_kernels.h"

#ifdef __CUDACC__
#define BG_HD_ORDER __host__ __device__ __forceinline__
#else
#define BG_HD_ORDER inline
#endif

namespace bg {

// Sample j of a batch (j < n) is pool entry ((base + j) * perm_mul + perm_add) mod n_total: with
// perm_mul coprime to n_total this visits the pool in a shuffled order, epoch by epoch.
struct PoolOrder {
    uint32_t n_total, perm_mul, perm_add, pad;
    BG_HD_ORDER uint32_t at(uint32_t j) const {
        return (uint32_t)(((uint64_t)j * perm_mul + perm_add) % n_total);
    }
};

struct GuideTrainArgs {
    const uint8_t* wpack;    // BF16 weight image
    const float4* samples;   // 4 float4 per sample (the whole pool)
    PoolOrder order;
    uint32_t base;           // first batch position
    uint32_t n;              // samples in this batch (rows past n are zero-weight)
    const float* wsum;       // sums of the batch's weights of head 0 and head 1 (two device floats)
    float alpha;             // loss blend, see guide_loss_grad
    float* partial;          // per-CTA gradient slices (>= ceil(n / 128) * GUIDE_PARAMS floats; entries
                             // of unused rows stay as they are: keep them zero)
    float* grad;             // FP32 gradient accumulator (GUIDE_PARAMS): += the sum of the slices
    float* stats;            // [0] += loss, [1] += samples with weight > 0
    uint32_t* step;          // Adam step counter, incremented once per launch (null: gradient only)
    uint32_t* err;           // error word
};

struct GuideAdam {
    float lr, beta1, beta2, eps;
};

// Forward pass over nranges (<= GUIDE_MAX_RANGES) ranges of queries: range r holds
// min(counts[r], stride) queries from index r * stride (counts: device, null = `stride` queries in
// every range).  out, at the same indices: raw outputs (GUIDE_RAW_STRIDE floats per query) or,
// with mixture, the parsed mixture records of both heads, head-major (head h's record of query q
// at (h * nranges * stride + q) * GUIDE_MIX_HEAD; out must be 16-byte aligned).
constexpr int GUIDE_MAX_RANGES = 3;
void launch_guide_infer(const uint8_t* wpack, const float4* query, const uint32_t* counts, uint32_t nranges,
                        uint32_t stride, float* out, bool mixture, uint32_t* err, int sms, cudaStream_t s);
// Forward + backward of a.n samples (one CTA per 128) and the reduction of their partial
// gradients into a.grad (two launches).
void launch_guide_train(const GuideTrainArgs& a, cudaStream_t s);
void launch_guide_adam(float* p, float* m, float* v, float* g, uint8_t* wpack, const uint32_t* step,
                       const GuideAdam& h, cudaStream_t s);
void launch_guide_pack(const float* p, uint8_t* wpack, cudaStream_t s);
// wsum[2b], wsum[2b + 1] = sums of the positive finite indirect (head 0) and direct (head 1)
// weights of batch b (positions b*batch .. in `order`).
void launch_guide_wsum(const float4* samples, const PoolOrder& order, uint32_t batch, float* wsum, cudaStream_t s);
// Relative variance of this pass's samples (film.pass) against the mean of the earlier passes:
// film.pass holds the sum of this pass's k samples per pixel.  With x = pass / k and m the mean of
// the n - k earlier samples, (x - m)^2 has expectation var (1/k + 1/(n - k)), so
// out[0] += sum over pixels with n > k and channels of (x - m)^2 / (m^2 + 0.01) / (1/k + 1/(n - k)),
// out[1] += number of terms: out[0] / out[1] estimates the relative variance of one sample.
void launch_pass_relvar(const FilmBuffers& film, uint32_t k, double* out, cudaStream_t s);
void launch_guide_mixture_eval(const float* raw, const float* u, const float* w, const float* pb, uint32_t n,
                               float alpha, float* out, cudaStream_t s);
// Limit of the network kernels' tensor-core waits on the current device, in SM clock cycles
// (0 or >= 2^31: the default, ~1 s).
cudaError_t set_guide_wait_limit(uint64_t cycles, cudaStream_t s);

}  // namespace bg

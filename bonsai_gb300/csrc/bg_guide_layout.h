// bg_guide_layout.h - layout constants of the guiding network, shared by host and device code.
//
// Biases are folded into the weights: every layer reads 80 input columns, one of which is a
// constant 1 (column 78 of the encoded input, column 64 of a hidden activation) whose weight is
// the bias.  Parameter layout (FP32 master copy, row-major W[out][80]):
//   layer 0..3: 64 rows at offset 5120 l; layer 4: 96 rows (82 used) at 20480; 28,160 floats.
// The output layer holds two heads of 41 outputs (8 vMF lobes + a selection logit each): head 0
// (rows 0..40) proposes the path's continuation and learns the radiance that arrives indirectly
// along a direction; head 1 (rows 41..81) proposes next-event directions and learns the emission
// a direction reaches directly.
// The tensor-core kernels read a BF16 image of the same weights, each layer tiled into 8x8
// core matrices (8-row groups 1280 B apart): 10,240 B per 64-row layer, 56,320 B in total.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define BG_LAYOUT_FN constexpr __host__ __device__
#else
#define BG_LAYOUT_FN constexpr
#endif

namespace bg {

constexpr int GUIDE_LAYERS = 5;
constexpr int GUIDE_K = 80;          // padded input width of every layer (incl. the bias column)
constexpr int GUIDE_HID = 64;
constexpr int GUIDE_HEADS = 2;
constexpr int GUIDE_HEAD_OUT = 41;   // per head: 8 lobes x (direction 3, log kappa, weight logit) + selection logit
constexpr int GUIDE_OUT = GUIDE_HEADS * GUIDE_HEAD_OUT;  // 82
constexpr int GUIDE_OUT_ROWS = 96;   // output rows padded to a multiple of 16 (and of 32)
constexpr int GUIDE_LOBES = 8;
constexpr int GUIDE_OCTAVES = 12;
constexpr int GUIDE_IN_USED = 78;
constexpr int GUIDE_PARAMS = 4 * GUIDE_HID * GUIDE_K + GUIDE_OUT_ROWS * GUIDE_K;  // 28,160
constexpr uint32_t GUIDE_ROWGROUP_BYTES = 8 * GUIDE_K * 2;                      // 1280
constexpr uint32_t GUIDE_WPACK_BYTES = (4 * GUIDE_HID + GUIDE_OUT_ROWS) * GUIDE_K * 2;  // 56,320
constexpr int GUIDE_RAW_STRIDE = 96;  // floats per query in the raw output buffer
// Mixture record of one head as the render-side inference stores it (floats): lobe i at 4i =
// kappa * mean direction (xyz) and log(weight) + log(normalisation) - kappa, so that the density is
// sum_i exp(m[4i+3] + m[4i..4i+2] . w); 32 + i (i < 7) = running sum of the lobe weights; 39 = c.
// Both heads per query (continuation head first), stored head-major: all queries' head-0 records,
// then all queries' head-1 records; GUIDE_MIX_STRIDE is the floats per query over both heads.
constexpr int GUIDE_MIX_HEAD = 40;
constexpr int GUIDE_MIX_STRIDE = GUIDE_HEADS * GUIDE_MIX_HEAD;  // 80
constexpr int GUIDE_QUERY_F4 = 3;     // query = 3 float4: p.xyz n.x | n.yz wo.xy | wo.z - - -
// training sample = query + wi.xyz (f2.yzw) + p_bsdf, indirect weight, direct weight (f3.xyz)
constexpr int GUIDE_SAMPLE_F4 = 4;

BG_LAYOUT_FN int guide_rows(int l) { return l == GUIDE_LAYERS - 1 ? GUIDE_OUT_ROWS : GUIDE_HID; }
BG_LAYOUT_FN int guide_used_rows(int l) { return l == GUIDE_LAYERS - 1 ? GUIDE_OUT : GUIDE_HID; }
BG_LAYOUT_FN int guide_param_off(int l) { return l * GUIDE_HID * GUIDE_K; }
BG_LAYOUT_FN uint32_t guide_wpack_off(int l) { return (uint32_t)l * GUIDE_HID * GUIDE_K * 2; }
BG_LAYOUT_FN int guide_bias_col(int l) { return l == 0 ? GUIDE_IN_USED : GUIDE_HID; }

}  // namespace bg

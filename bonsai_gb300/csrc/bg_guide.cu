// bg_guide.cu - tensor-core kernels of the guiding network (tcgen05, BF16 operands in shared
// memory, FP32 accumulators in TMEM) and its optimiser.
//
//   k_guide_infer  forward pass for a queue of queries, 128 queries per tile (one per thread /
//                  TMEM lane); persistent CTAs keep the 48.6 KB weight image in shared memory.
//   k_guide_train  fused forward + loss gradient + backward for 128 training samples per CTA:
//                  activations of all layers stay in shared memory, dX = dZ W and
//                  dW = dZ^T H run as MN-major MMAs on the same tiles, each CTA stores its weight
//                  gradient (plain stores, no atomics) into its slice of a partial buffer.
//   k_guide_reduce sums the CTAs' partial gradients into the FP32 gradient.
//   k_guide_adam   Adam on the FP32 master weights; rewrites the BF16 core-matrix image.
// Both network kernels bring the weight image into shared memory with one bulk (TMA) copy.
//
// Shared-memory tiles (no swizzle, core matrices of 8 rows x 16 B, see bg_umma.cuh):
//   weights  W_l[rows][80]  8-row groups 1280 B apart      (56,320 B for all five layers)
//   act      A[128][80]     8-row groups 1280 B apart      (20,480 B per layer)
//   dZ       dZ[128][128]   8-row groups 2048 B apart; dZ^T feeds an M = 128 MMA for layers with
//            64 (or 96) output rows: the dW rows past a layer's outputs are computed and dropped.
// TMEM columns: forward accumulator 0..95; backward dW 0..79 (the forward accumulator is free by
// then) and dX 128..207 (training allocates 256 columns, inference 128).
#include <cuda_bf16.h>

#include "bg_device.h"
#include "bg_guide.cuh"
#include "bg_guide_kernels.h"
#include "bg_umma.cuh"

namespace bg {

// Limit (SM clock cycles) of the first wait on each MMA stage; bail_out's drain wait always uses
// the default, so MMAs in flight retire before TMEM is freed.  Set by set_guide_wait_limit.
__device__ long long g_guide_wait_limit = kWaitLimitCycles;

namespace {

constexpr uint32_t ACT_BYTES = 128 * GUIDE_K * 2;         // 20,480
constexpr uint32_t ACT_RS = GUIDE_ROWGROUP_BYTES;         // 1280
constexpr uint32_t DZ_RS = 2048;                          // 16 column groups per 8-row group
constexpr uint32_t DZ_BYTES = 16 * DZ_RS;                 // 32,768
constexpr int INFER_WG = 2;  // warpgroups (tiles in flight) per inference CTA
constexpr uint32_t INFER_TM_COLS = 128 * INFER_WG;
constexpr uint32_t INFER_SMEM = GUIDE_WPACK_BYTES + INFER_WG * ACT_BYTES;  // 97,280: weights + one tile per warpgroup
constexpr uint32_t TRAIN_SMEM = GUIDE_WPACK_BYTES + 5 * ACT_BYTES + DZ_BYTES;          // 191,488
constexpr uint32_t TM_FWD = 0, TM_DW = 0, TM_DX = 128, TM_COLS_TRAIN = 256, TM_COLS_INFER = 128;  // per tile
static_assert(GUIDE_OUT_ROWS <= (int)TM_DX && TM_DX + GUIDE_K <= TM_COLS_TRAIN, "TMEM column plan");
static_assert(GUIDE_OUT_ROWS <= (int)TM_COLS_INFER && GUIDE_HID <= (int)TM_COLS_INFER, "TMEM column plan");

BG_D uint32_t pack_bf16(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}
BG_D float bf16_lo(uint32_t u) { return __uint_as_float(u << 16); }
BG_D float bf16_hi(uint32_t u) { return __uint_as_float(u & 0xFFFF0000u); }

// Writes 8 consecutive columns (c0 a multiple of 8) of one row.
BG_D void store_row8(uint8_t* tile, uint32_t rs, uint32_t row, uint32_t c0, const float* v) {
    uint4 q = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
    *reinterpret_cast<uint4*>(tile + core_off(row, c0, rs)) = q;
}

// Encoded query -> one row of an activation tile (80 columns).
BG_D void encode_row(uint8_t* act, uint32_t row, const float* q) {
    float x[GUIDE_K];
    guide_encode(q, x);
#pragma unroll
    for (int g = 0; g < GUIDE_K / 8; ++g) store_row8(act, ACT_RS, row, 8 * g, x + 8 * g);
}

// D[tm] = act (128 x 80, K-major) * W_l^T (N x 80, K-major); five K = 16 steps.
BG_D void issue_forward(uint32_t tm, uint32_t act, uint32_t w, int N) {
#pragma unroll
    for (int k = 0; k < GUIDE_K / 16; ++k)
        umma_bf16(tm, umma_desc(act + 256 * k, 128, ACT_RS), umma_desc(w + 256 * k, 128, ACT_RS),
                  umma_idesc_bf16(128, N, 0, 0), k > 0);
}

// Forward epilogue of a hidden layer: ReLU of this thread's 64 accumulator columns, BF16, plus
// the constant bias column 64 and zero columns 65..79.
BG_D void hidden_epilogue(uint32_t tm_row, uint8_t* dst, uint32_t row) {
    float v[GUIDE_HID];
    tmem_ld64(tm_row, v);  // one TMEM round trip for the row's 64 accumulators
#pragma unroll
    for (int j = 0; j < GUIDE_HID; ++j) v[j] = fmaxf(v[j], 0.0f);
#pragma unroll
    for (int c = 0; c < GUIDE_HID; c += 8) store_row8(dst, ACT_RS, row, c, v + c);
    float tail[16] = {1.0f};
    store_row8(dst, ACT_RS, row, 64, tail);
    store_row8(dst, ACT_RS, row, 72, tail + 8);
}

// Closes an MMA stage: makes this thread's shared-memory writes visible to the tensor core and
// orders TMEM reads before the next MMA.  Returns true when any thread saw a timeout.
BG_D bool stage_barrier(bool ok) {
    fence_async_smem();
    tc_fence_before();
    int bad = __syncthreads_or(!ok);
    tc_fence_after();
    return bad != 0;
}

// Bounded clean-up after a timed-out wait: records the error, lets the in-flight MMAs retire
// (again with a limit) and frees TMEM.
BG_D void bail_out(uint64_t* bar, uint32_t parity, uint32_t* err, uint32_t tmem, uint32_t ncols) {
    if (threadIdx.x == 0) atomicOr(err, ERR_GUIDE_TIMEOUT);
    mbar_wait(bar, parity);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32) tmem_dealloc(tmem, ncols);
}

}  // namespace

// ---------------------------------------------------------------- inference
// MIX = false: the 82 raw outputs per query (GUIDE_RAW_STRIDE floats); MIX = true: the parsed
// mixture records of both heads that the render kernels sample, head-major: head h's record of
// query q at (h * nranges * stride + q) * GUIDE_MIX_HEAD.
// Queries come in `nranges` ranges: range r holds min(counts[r], stride) queries from r * stride
// (counts null: one range of `stride` queries); outputs use the same indices.
// Each CTA runs INFER_WG warpgroups, each on its own tile of 128 queries (one per thread / TMEM
// lane) with its own TMEM accumulator (128 columns), activation tile (updated in place: a layer's
// epilogue overwrites the tile its MMA has finished reading), mbarrier and named barrier, so the
// tensor core works on one warpgroup's layer while the other runs an epilogue.  The weight image
// in shared memory is loaded once per CTA and shared.

// Named barrier ID (1.., 0 is __syncthreads) over the 128 threads of one warpgroup, with an OR of
// `pred` (the ID is an immediate, so the kernel reserves only the barriers it names).
template <int ID>
BG_D bool wg_sync_or(bool pred) {
    uint32_t r;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.u32 q, %1, 0;\nbar.red.or.pred p, %2, 128, q;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)pred), "n"(ID)
        : "memory");
    return r != 0;
}
// Stage barrier of warpgroup wg (see stage_barrier).
BG_D bool wg_stage_barrier(bool ok, uint32_t wg) {
    static_assert(INFER_WG == 2, "one named barrier per warpgroup");
    fence_async_smem();
    tc_fence_before();
    bool bad = wg == 0 ? wg_sync_or<1>(!ok) : wg_sync_or<2>(!ok);
    tc_fence_after();
    return bad;
}

template <bool MIX>
__global__ void __launch_bounds__(128 * INFER_WG, 2) k_guide_infer(const uint8_t* wpack, const float4* query,
                                                                  const uint32_t* counts, uint32_t nranges,
                                                                  uint32_t stride, float* raw, uint32_t* err) {
    extern __shared__ __align__(128) uint8_t sm[];
    __shared__ uint64_t bar[INFER_WG], wbar;
    __shared__ uint32_t tslot;
    uint32_t rn[GUIDE_MAX_RANGES], rt[GUIDE_MAX_RANGES + 1];  // queries and first tile of each range
    rt[0] = 0;
#pragma unroll
    for (int r = 0; r < GUIDE_MAX_RANGES; ++r) {
        rn[r] = (uint32_t)r < nranges ? (counts ? min(counts[r], stride) : stride) : 0u;
        rt[r + 1] = rt[r] + (rn[r] + 127) / 128;
    }
    const uint32_t ntiles = rt[GUIDE_MAX_RANGES];
    if (blockIdx.x * INFER_WG >= ntiles) return;  // uniform over the CTA, before any barrier
    const long long wait_limit = g_guide_wait_limit;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, wg = tid >> 7, wtid = tid & 127u;
    uint8_t* wsm = sm;
    uint8_t* act = sm + GUIDE_WPACK_BYTES + wg * ACT_BYTES;
    if (tid == 0) {
        for (int k = 0; k < INFER_WG; ++k) mbar_init(&bar[k], 1);
        mbar_init(&wbar, 1);
    }
    if (warp == 0) tmem_alloc(&tslot, INFER_TM_COLS);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) bulk_g2s(wsm, wpack, GUIDE_WPACK_BYTES, &wbar);
    if (__syncthreads_or(!mbar_wait(&wbar, 0, wait_limit))) {
        // the weight copy did not arrive in time: record it, let it land (default limit) and stop
        if (tid == 0) atomicOr(err, ERR_GUIDE_TIMEOUT);
        mbar_wait(&wbar, 0);
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (warp == 0) tmem_dealloc(tslot, INFER_TM_COLS);
        return;
    }
    const uint32_t tmem = tslot + 128u * wg;                  // this warpgroup's columns
    const uint32_t tm_row = tmem + (((warp & 3u) * 32u) << 16);  // this warp's lane quarter
    const uint32_t w_addr = smem_addr(wsm), a_addr = smem_addr(act);
    uint32_t phase = 0;
    // this thread's query of a tile: index, and whether the tile holds one for its row
    // (and the tile's number of queries, rows 0 .. rows - 1)
    auto locate = [&](uint32_t tile, uint32_t& qi, uint32_t& rows) {
        uint32_t r = 0;
#pragma unroll
        for (int j = 1; j < GUIDE_MAX_RANGES; ++j)
            if (tile >= rt[j]) r = j;
        const uint32_t local = (tile - rt[r]) * 128 + wtid;
        qi = r * stride + local;
        rows = min(128u, rn[r] - (tile - rt[r]) * 128);
        return local < rn[r];
    };
    // the next tile's query is loaded while this tile's layers run
    const uint32_t tstep = gridDim.x * INFER_WG;
    uint32_t tile = blockIdx.x * INFER_WG + wg, qi = 0, rows = 0;
    bool valid = locate(tile, qi, rows);
    // head h's records follow those of head h - 1 (head-major), GUIDE_MIX_HEAD floats per query
    const size_t head_stride = (size_t)nranges * stride * GUIDE_MIX_HEAD;
    float4 qa = make_float4(0.5f, 0.5f, 0.5f, 0.0f), qb = make_float4(0.0f, 1.0f, 0.0f, 0.0f),
           qc = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
    if (valid) {
        qa = query[3 * (size_t)qi];
        qb = query[3 * (size_t)qi + 1];
        qc = query[3 * (size_t)qi + 2];
    }
    for (; tile < ntiles; tile += tstep) {
        float q[9] = {qa.x, qa.y, qa.z, qa.w, qb.x, qb.y, qb.z, qb.w, qc.x};
        encode_row(act, wtid, q);
        const uint32_t cur_qi = qi, cur_rows = rows;
        const bool cur_valid = valid;
        valid = tile + tstep < ntiles && locate(tile + tstep, qi, rows);
        if (valid) {
            qa = query[3 * (size_t)qi];
            qb = query[3 * (size_t)qi + 1];
            qc = query[3 * (size_t)qi + 2];
        }
        wg_stage_barrier(true, wg);  // no wait before the first stage
        bool stop = false;
        for (int l = 0; l < GUIDE_LAYERS; ++l) {
            const int N = guide_rows(l);
            if (wtid == 0) {
                issue_forward(tmem + TM_FWD, a_addr, w_addr + guide_wpack_off(l), N);
                umma_commit(&bar[wg]);
            }
            bool ok = mbar_wait(&bar[wg], phase, wait_limit);
            phase ^= 1;
            tc_fence_after();
            if (l < GUIDE_LAYERS - 1) {
                hidden_epilogue(tm_row + TM_FWD, act, wtid);
            } else if (MIX) {
                // Each head's records go through the activation tile (free once the last MMA has
                // read it: 128 rows x 160 B = ACT_BYTES) and leave in one bulk copy of the tile's
                // rows, which hold its queries contiguously from row 0.
#pragma unroll
                for (int h = 0; h < GUIDE_HEADS; ++h) {
                    // head h's 41 outputs from the 48 or 64 columns that hold them
                    float v[64];
                    const int c0 = h == 0 ? 0 : 32;
                    if (h == 0) {
                        tmem_ld32(tm_row + TM_FWD, v);
                        tmem_ld16(tm_row + TM_FWD + 32, v + 32);
                    } else {
                        tmem_ld64(tm_row + TM_FWD + 32, v);
                    }
                    if (cur_valid) {
                        float rec[GUIDE_MIX_HEAD];
                        guide_write_mixture(v + (GUIDE_HEAD_OUT * h - c0), rec);
                        float4* o = reinterpret_cast<float4*>(act + wtid * (GUIDE_MIX_HEAD * 4));
#pragma unroll
                        for (int j = 0; j < GUIDE_MIX_HEAD / 4; ++j)
                            o[j] = make_float4(rec[4 * j], rec[4 * j + 1], rec[4 * j + 2], rec[4 * j + 3]);
                    }
                    fence_async_smem();
                    if (wg == 0) wg_sync_or<1>(false);
                    else wg_sync_or<2>(false);
                    if (wtid == 0) {
                        bulk_s2g(raw + h * head_stride + (size_t)(cur_qi - wtid) * GUIDE_MIX_HEAD, act,
                                 cur_rows * (GUIDE_MIX_HEAD * 4));
                        bulk_wait_read();  // the tile is rewritten next (the other head, or the next encode)
                    }
                    if (h + 1 < GUIDE_HEADS) {
                        if (wg == 0) wg_sync_or<1>(false);
                        else wg_sync_or<2>(false);
                    }
                }
            } else {
#pragma unroll
                for (int c = 0; c < GUIDE_OUT_ROWS; c += 32) {
                    float v[32];
                    tmem_ld32(tm_row + TM_FWD + c, v);
                    if (cur_valid) {
                        float4* o = reinterpret_cast<float4*>(raw + (size_t)cur_qi * GUIDE_RAW_STRIDE + c);
#pragma unroll
                        for (int j = 0; j < 8; ++j) o[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                    }
                }
            }
            if (wg_stage_barrier(ok, wg)) {
                // a wait ran out: record it, let this warpgroup's issued MMAs retire (default
                // limit) and stop; TMEM is freed once both warpgroups are done
                if (wtid == 0) atomicOr(err, ERR_GUIDE_TIMEOUT);
                mbar_wait(&bar[wg], phase ^ 1);
                stop = true;
                break;
            }
        }
        if (stop) break;
    }
    if (MIX && wtid == 0) bulk_wait_all();  // this warpgroup's record copies have landed
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tslot, INFER_TM_COLS);
}

// ---------------------------------------------------------------- training
// 256 threads per 128-sample tile: thread t serves row t % 128 (its TMEM lane, warp % 4 selecting
// the lane quarter) and half t / 128 of the row's columns in every epilogue, so each stage's
// epilogue (TMEM loads, activation / gradient packing, shared-memory and gradient stores) takes
// half the time of one thread per row.  The output layer splits by head: half 0 takes the
// continuation head's loss, half 1 the next-event head's (their dZ columns 40 and 41..47 share an
// 8-column group, assembled through `xch`).
__global__ void __launch_bounds__(256, 1) k_guide_train(GuideTrainArgs a) {
    extern __shared__ __align__(128) uint8_t sm[];
    __shared__ uint64_t bar, wbar;
    __shared__ uint32_t tslot;
    __shared__ float xch[128];  // head 0's gradient of output 40, per row
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t row = tid & 127u, half = tid >> 7;
    const long long wait_limit = g_guide_wait_limit;
    if (a.step && blockIdx.x == 0 && tid == 0) atomicAdd(a.step, 1u);
    uint8_t* wsm = sm;
    uint8_t* act = sm + GUIDE_WPACK_BYTES;  // 5 tiles: X0, H1..H4
    uint8_t* dz = sm + GUIDE_WPACK_BYTES + 5 * ACT_BYTES;
    {   // zero dZ (columns past a layer's outputs must read as finite values in every dW MMA)
        uint4* d = reinterpret_cast<uint4*>(dz);
        for (uint32_t i = tid; i < DZ_BYTES / 16; i += blockDim.x) d[i] = make_uint4(0, 0, 0, 0);
    }
    if (tid == 0) {
        mbar_init(&bar, 1);
        mbar_init(&wbar, 1);
    }
    if (warp == 0) tmem_alloc(&tslot, TM_COLS_TRAIN);
    __syncthreads();  // the barriers are initialised before the bulk copy signals one
    if (tid == 0) bulk_g2s(wsm, a.wpack, GUIDE_WPACK_BYTES, &wbar);
    // this row's sample (both halves read it; half 0 encodes it)
    const uint32_t si = blockIdx.x * 128 + row;
    float q[9] = {0.5f, 0.5f, 0.5f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 1.0f};
    V3 wi = v3(0.0f, 0.0f, 1.0f);
    float p_b = 0.0f, wn = 0.0f;  // this half's head: its normalised weight
    bool any_w = false;
    if (si < a.n) {
        const float4* s = a.samples + (size_t)GUIDE_SAMPLE_F4 * a.order.at(a.base + si);
        float4 f0 = s[0], f1 = s[1], f2 = s[2], f3 = s[3];
        q[0] = f0.x; q[1] = f0.y; q[2] = f0.z; q[3] = f0.w; q[4] = f1.x; q[5] = f1.y; q[6] = f1.z; q[7] = f1.w;
        q[8] = f2.x;
        wi = v3(f2.y, f2.z, f2.w);
        p_b = f3.x;
        const float ws0 = a.wsum[0], ws1 = a.wsum[1];
        const float wn0 = (ws0 > 0.0f && f3.y > 0.0f && isfinite(f3.y)) ? f3.y / ws0 : 0.0f;
        const float wn1 = (ws1 > 0.0f && f3.z > 0.0f && isfinite(f3.z)) ? f3.z / ws1 : 0.0f;
        wn = half == 0 ? wn0 : wn1;
        any_w = wn0 > 0.0f || wn1 > 0.0f;
    }
    if (half == 0) encode_row(act, row, q);
    const bool wok = mbar_wait(&wbar, 0, wait_limit);  // the weight image (overlaps the encoding above)
    fence_async_smem();
    tc_fence_before();
    const bool wbad = __syncthreads_or(!wok);
    tc_fence_after();
    if (wbad) {
        if (tid == 0) atomicOr(a.err, ERR_GUIDE_TIMEOUT);
        mbar_wait(&wbar, 0);
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (warp == 0) tmem_dealloc(tslot, TM_COLS_TRAIN);
        return;
    }
    const uint32_t tmem = tslot;
    const uint32_t tm_row = tmem + (((warp & 3u) * 32u) << 16);
    const uint32_t w_addr = smem_addr(wsm), act_addr = smem_addr(act), dz_addr = smem_addr(dz);
    const float zero8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    uint32_t phase = 0;
    // forward
    for (int l = 0; l < GUIDE_LAYERS; ++l) {
        if (tid == 0) {
            issue_forward(tmem + TM_FWD, act_addr + l * ACT_BYTES, w_addr + guide_wpack_off(l), guide_rows(l));
            umma_commit(&bar);
        }
        bool ok = mbar_wait(&bar, phase, wait_limit);
        phase ^= 1;
        tc_fence_after();
        if (l < GUIDE_LAYERS - 1) {
            // ReLU of this half's 32 accumulator columns -> BF16; half 1 adds the bias column 64
            // (constant 1) and the zero columns 65..79
            uint8_t* dst = act + (l + 1) * ACT_BYTES;
            const uint32_t c0 = 32u * half;
            float v[32];
            tmem_ld32(tm_row + TM_FWD + c0, v);
#pragma unroll
            for (int j = 0; j < 32; ++j) v[j] = fmaxf(v[j], 0.0f);
#pragma unroll
            for (int c = 0; c < 32; c += 8) store_row8(dst, ACT_RS, row, c0 + c, v + c);
            if (half == 1) {
                float tail[16] = {1.0f};
                store_row8(dst, ACT_RS, row, 64, tail);
                store_row8(dst, ACT_RS, row, 72, tail + 8);
            }
        } else {
            // this half's head: 41 outputs from the 48 (head 0) or 64 (head 1) columns holding them
            float v[64], g[GUIDE_HEAD_OUT];
            if (half == 0) {
                tmem_ld32(tm_row + TM_FWD, v);
                tmem_ld16(tm_row + TM_FWD + 32, v + 32);
            } else {
                tmem_ld64(tm_row + TM_FWD + 32, v);
            }
            // head 1's outputs start at v[9] (column 41); constant offsets keep v in registers
            float loss = half == 0 ? guide_loss_grad(v, wi, p_b, wn, a.alpha, g)
                                   : guide_loss_grad(v + (GUIDE_HEAD_OUT - 32), wi, p_b, wn, a.alpha, g);
            // loss gradient -> dZ4: head 0 in columns 0..40, head 1 in 41..81, 82..127 zero
            if (half == 0) {
#pragma unroll
                for (int c = 0; c < 40; c += 8) store_row8(dz, DZ_RS, row, c, g + c);
                xch[row] = g[40];
            }
            __syncthreads();  // xch
            if (half == 1) {
                float b[8] = {xch[row], g[0], g[1], g[2], g[3], g[4], g[5], g[6]};
                store_row8(dz, DZ_RS, row, 40, b);
#pragma unroll
                for (int c = 48; c < 88; c += 8) {
                    float t[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) t[j] = c + j - 41 < GUIDE_HEAD_OUT ? g[c + j - 41] : 0.0f;
                    store_row8(dz, DZ_RS, row, c, t);
                }
#pragma unroll
                for (int c = 88; c < 128; c += 8) store_row8(dz, DZ_RS, row, c, zero8);
            }
            float cnt = half == 0 && any_w ? 1.0f : 0.0f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                loss += __shfl_xor_sync(0xffffffffu, loss, o);
                cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
            }
            if (lane == 0) {
                atomicAdd(&a.stats[0], loss);
                if (half == 0) atomicAdd(&a.stats[1], cnt);
            }
        }
        if (stage_barrier(ok)) {
            bail_out(&bar, phase ^ 1, a.err, tmem, TM_COLS_TRAIN);
            return;
        }
    }
    // backward: layer l's dZ is in `dz`; its input activation is act tile l
    for (int l = GUIDE_LAYERS - 1; l >= 0; --l) {
        const uint32_t a_l = act_addr + l * ACT_BYTES;
        const uint32_t w_l = w_addr + guide_wpack_off(l);
        const int kout = guide_rows(l);  // 96 or 64 dZ columns feed the dX MMA
        if (tid == 0) {
            if (l > 0) {
                // dX = dZ (128 x kout, K-major) * W_l (kout x 80 read MN-major: N = 80 input columns)
                for (int k = 0; k < kout / 16; ++k)
                    umma_bf16(tmem + TM_DX, umma_desc(dz_addr + 256 * k, 128, DZ_RS),
                              umma_desc(w_l + 2 * ACT_RS * k, ACT_RS, 128), umma_idesc_bf16(128, GUIDE_K, 0, 1),
                              k > 0);
            }
            // dW = dZ^T (M = 128 output rows incl. zero rows, K = 128 samples) * act_l (N = 80, K = samples)
            for (int k = 0; k < 128 / 16; ++k)
                umma_bf16(tmem + TM_DW, umma_desc(dz_addr + 2 * DZ_RS * k, DZ_RS, 128),
                          umma_desc(a_l + 2 * ACT_RS * k, ACT_RS, 128), umma_idesc_bf16(128, GUIDE_K, 1, 1), k > 0);
            umma_commit(&bar);
        }
        bool ok = mbar_wait(&bar, phase, wait_limit);
        phase ^= 1;
        tc_fence_after();
        // weight gradient rows (row = output row) into this CTA's partial slice: half 0 takes
        // columns 0..47, half 1 columns 48..79
        const int used = guide_used_rows(l);
        if ((int)((warp & 3u) * 32) < used) {
            float4* gl = reinterpret_cast<float4*>(a.partial + (size_t)blockIdx.x * GUIDE_PARAMS + guide_param_off(l) +
                                                   row * GUIDE_K);
            float v[48];
            const int c0 = half == 0 ? 0 : 48, nc = half == 0 ? 48 : 32;
            if (half == 0) {
                tmem_ld32(tm_row + TM_DW, v);
                tmem_ld16(tm_row + TM_DW + 32, v + 32);
            } else {
                tmem_ld32(tm_row + TM_DW + 48, v);
            }
            if ((int)row < used) {
#pragma unroll
                for (int j = 0; j < 12; ++j)
                    if (4 * j < nc) gl[c0 / 4 + j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
            }
        }
        if (l > 0) {
            // dZ_{l-1} = dX[:, 0..63] * relu'(H_l), H_l = act tile l (this row; this half's 32 columns)
            const uint8_t* hrow = act + l * ACT_BYTES;
            const int c0 = 32 * (int)half;
            float v[32];
            tmem_ld32(tm_row + TM_DX + c0, v);
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                uint4 hv = *reinterpret_cast<const uint4*>(hrow + core_off(row, c0 + 8 * h, ACT_RS));
                uint32_t hw[4] = {hv.x, hv.y, hv.z, hv.w};
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (!(bf16_lo(hw[j]) > 0.0f)) v[8 * h + 2 * j] = 0.0f;
                    if (!(bf16_hi(hw[j]) > 0.0f)) v[8 * h + 2 * j + 1] = 0.0f;
                }
            }
#pragma unroll
            for (int c = 0; c < 32; c += 8) store_row8(dz, DZ_RS, row, c0 + c, v + c);
        }
        if (stage_barrier(ok)) {
            bail_out(&bar, phase ^ 1, a.err, tmem, TM_COLS_TRAIN);
            return;
        }
    }
    if (warp == 0) tmem_dealloc(tmem, TM_COLS_TRAIN);
}

// ---------------------------------------------------------------- optimiser and helpers
__device__ __forceinline__ void pack_param(uint8_t* wpack, int i, float p) {
    int l = min(i / (GUIDE_HID * GUIDE_K), GUIDE_LAYERS - 1);
    int r = (i - guide_param_off(l)) / GUIDE_K, c = (i - guide_param_off(l)) % GUIDE_K;
    *reinterpret_cast<__nv_bfloat16*>(wpack + guide_wpack_off(l) + core_off(r, c, ACT_RS)) = __float2bfloat16_rn(p);
}

__global__ void k_guide_adam(float* p, float* m, float* v, float* g, uint8_t* wpack, const uint32_t* step,
                             GuideAdam h) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= GUIDE_PARAMS) return;
    float gi = g[i];
    g[i] = 0.0f;
    float t = (float)max(*step, 1u);
    float mi = h.beta1 * m[i] + (1.0f - h.beta1) * gi;
    float vi = h.beta2 * v[i] + (1.0f - h.beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float mhat = mi / (1.0f - powf(h.beta1, t));
    float vhat = vi / (1.0f - powf(h.beta2, t));
    float pi = p[i] - h.lr * mhat / (sqrtf(vhat) + h.eps);
    p[i] = pi;
    pack_param(wpack, i, pi);
}

// grad[i] += sum over the n CTAs' partial gradients (parameter i of slice b at b * GUIDE_PARAMS + i).
// blockIdx.y takes every REDUCE_SPLIT-th slice, so REDUCE_SPLIT threads share a parameter (more
// loads in flight than one thread walking all slices); they add into grad atomically.
constexpr uint32_t REDUCE_SPLIT = 8;
__global__ void k_guide_reduce(const float* __restrict__ partial, uint32_t n, float* grad) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint32_t)GUIDE_PARAMS) return;
    float s0 = 0.0f, s1 = 0.0f;
    uint32_t b = blockIdx.y;
    for (; b + REDUCE_SPLIT < n; b += 2 * REDUCE_SPLIT) {
        s0 += partial[(size_t)b * GUIDE_PARAMS + i];
        s1 += partial[(size_t)(b + REDUCE_SPLIT) * GUIDE_PARAMS + i];
    }
    if (b < n) s0 += partial[(size_t)b * GUIDE_PARAMS + i];
    const float s = s0 + s1;
    if (s != 0.0f) atomicAdd(&grad[i], s);
}

__global__ void k_guide_pack(const float* p, uint8_t* wpack) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < GUIDE_PARAMS) pack_param(wpack, i, p[i]);
}

// Sums of the two heads' training weights of each batch of the sample pool (wsum[2b], wsum[2b + 1]).
__global__ void k_guide_wsum(const float4* samples, PoolOrder order, uint32_t batch, float* wsum) {
    __shared__ float2 red[256];
    const uint32_t b0 = blockIdx.x * batch, b1 = min(order.n_total, b0 + batch);
    float2 s = make_float2(0.0f, 0.0f);
    for (uint32_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
        const float4 f3 = samples[(size_t)GUIDE_SAMPLE_F4 * order.at(i) + 3];
        if (f3.y > 0.0f && isfinite(f3.y)) s.x += f3.y;
        if (f3.z > 0.0f && isfinite(f3.z)) s.y += f3.z;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            red[threadIdx.x].x += red[threadIdx.x + o].x;
            red[threadIdx.x].y += red[threadIdx.x + o].y;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        wsum[2 * blockIdx.x] = red[0].x;
        wsum[2 * blockIdx.x + 1] = red[0].y;
    }
}

__global__ void k_pass_relvar(const double* sum, const uint32_t* count, const float* pass, uint32_t npix, uint32_t k,
                              double* out) {
    double acc = 0.0, cnt = 0.0;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
        const uint32_t n = count[p];
        if (n <= k) continue;
        const double scale = 1.0 / (1.0 / k + 1.0 / (double)(n - k));
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double x = (double)pass[3 * p + c] / k;
            const double m = (sum[3 * p + c] - pass[3 * p + c]) / (double)(n - k);
            const double d = x - m;
            acc += d * d / (m * m + 0.01) * scale;
            cnt += 1.0;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    if ((threadIdx.x & 31) == 0 && cnt > 0.0) {
        atomicAdd(&out[0], acc);
        atomicAdd(&out[1], cnt);
    }
}

// Test entry: mixture parsing, sampling, pdf and loss gradient for given raw outputs of one head.
// out (48 per item): sampled wi.xyz, pdf(sampled), pdf(w), c, loss, -, grad[40..] -> out[8..48]
__global__ void k_guide_mixture_eval(const float* raw, const float* u, const float* w, const float* pb, uint32_t n,
                                     float alpha, float* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float r[GUIDE_HEAD_OUT];
    for (int j = 0; j < GUIDE_HEAD_OUT; ++j) r[j] = raw[(size_t)GUIDE_HEAD_OUT * i + j];
    // the render path: stored mixture record read through MixView
    float rec[GUIDE_MIX_HEAD];
    guide_write_mixture(r, rec);
    const MixView m{rec};
    V3 ws = m.sample(u[3 * i], u[3 * i + 1], u[3 * i + 2]);
    V3 wq = v3(w[3 * i], w[3 * i + 1], w[3 * i + 2]);
    float g[GUIDE_HEAD_OUT];
    float loss = guide_loss_grad(r, wq, pb[i], 1.0f, alpha, g);
    float* o = out + (size_t)48 * i;
    o[0] = ws.x;
    o[1] = ws.y;
    o[2] = ws.z;
    o[3] = m.pdf(ws);
    o[4] = m.pdf(wq);
    o[5] = m.c();
    o[6] = loss;
    o[7] = 0.0f;
    for (int j = 0; j < 40; ++j) o[8 + j] = g[j];
    // g[40] (selection logit) goes in slot 7
    o[7] = g[40];
}

// ---------------------------------------------------------------- launchers
void guide_set_smem_limits() {
    static bool done = false;
    if (done) return;
    cudaFuncSetAttribute(k_guide_infer<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, INFER_SMEM);
    cudaFuncSetAttribute(k_guide_infer<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, INFER_SMEM);
    cudaFuncSetAttribute(k_guide_train, cudaFuncAttributeMaxDynamicSharedMemorySize, TRAIN_SMEM);
    done = true;
}

void launch_guide_infer(const uint8_t* wpack, const float4* query, const uint32_t* counts, uint32_t nranges,
                        uint32_t stride, float* out, bool mixture, uint32_t* err, int sms, cudaStream_t s) {
    if (nranges == 0 || nranges > (uint32_t)GUIDE_MAX_RANGES) return;
    guide_set_smem_limits();
    uint64_t tiles = (uint64_t)nranges * ((stride + 127) / 128);
    uint32_t grid = (uint32_t)std::min<uint64_t>((tiles + INFER_WG - 1) / INFER_WG, (uint64_t)sms * 2);
    if (grid == 0) return;
    if (mixture) k_guide_infer<true><<<grid, 128 * INFER_WG, INFER_SMEM, s>>>(wpack, query, counts, nranges, stride, out, err);
    else k_guide_infer<false><<<grid, 128 * INFER_WG, INFER_SMEM, s>>>(wpack, query, counts, nranges, stride, out, err);
}

void launch_guide_train(const GuideTrainArgs& a, cudaStream_t s) {
    guide_set_smem_limits();
    uint32_t grid = (a.n + 127) / 128;
    if (grid == 0) return;
    k_guide_train<<<grid, 256, TRAIN_SMEM, s>>>(a);
    k_guide_reduce<<<dim3((GUIDE_PARAMS + 255) / 256, REDUCE_SPLIT), 256, 0, s>>>(a.partial, grid, a.grad);
}

void launch_guide_adam(float* p, float* m, float* v, float* g, uint8_t* wpack, const uint32_t* step,
                       const GuideAdam& h, cudaStream_t s) {
    k_guide_adam<<<(GUIDE_PARAMS + 255) / 256, 256, 0, s>>>(p, m, v, g, wpack, step, h);
}

void launch_guide_pack(const float* p, uint8_t* wpack, cudaStream_t s) {
    k_guide_pack<<<(GUIDE_PARAMS + 255) / 256, 256, 0, s>>>(p, wpack);
}

void launch_guide_wsum(const float4* samples, const PoolOrder& order, uint32_t batch, float* wsum, cudaStream_t s) {
    uint32_t nb = (order.n_total + batch - 1) / batch;
    if (nb) k_guide_wsum<<<nb, 256, 0, s>>>(samples, order, batch, wsum);
}

void launch_pass_relvar(const FilmBuffers& film, uint32_t k, double* out, cudaStream_t s) {
    if (film.npix && film.pass && k) k_pass_relvar<<<1216, 256, 0, s>>>(film.sum, film.count, film.pass, film.npix, k, out);
}

void launch_guide_mixture_eval(const float* raw, const float* u, const float* w, const float* pb, uint32_t n,
                               float alpha, float* out, cudaStream_t s) {
    if (n) k_guide_mixture_eval<<<(n + 127) / 128, 128, 0, s>>>(raw, u, w, pb, n, alpha, out);
}

cudaError_t set_guide_wait_limit(uint64_t cycles, cudaStream_t s) {
    const long long v = (cycles == 0 || cycles >= (uint64_t)kWaitLimitCycles) ? kWaitLimitCycles : (long long)cycles;
    cudaError_t e = cudaMemcpyToSymbolAsync(g_guide_wait_limit, &v, sizeof(v), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // v lives on this stack frame
    return e;
}

}  // namespace bg

// tc_conv.cu -- convolution layers as implicit GEMMs on the tcgen05 tensor
// cores (BF16 operands, FP32 accumulators in TMEM).
//
// Reference: convolve<k,C,O> (Network.cpp:345-393) computes
//   out[o][p] = act(b[o] + sum_{c,ky,kx} W[o][c][ky][kx] * in[c][p + (ky,kx)])
// through an im2col matrix and one sgemm per layer.  Here the im2col never
// exists: activations live in HBM as "flat rows" (lg_common.cuh, layouts L3
// and L5) in which every tap of the filter is one constant row shift.  For a
// tile of 128 consecutive rows, one TMA load brings the tile plus its halo
// (the "window") into shared memory, and the A operand of tap t is the same
// window read through a shared-memory descriptor that starts
// (window_pre + shift_t) rows in.  The 128-byte swizzle is a function of the
// absolute shared-memory address, so a descriptor may start at any row; the
// window is loaded once and read by all 9 (or 5) taps.
//
// Per CTA (persistent, one per SM):
//   warp 0        TMA producer: windows (double-buffered) and weight slices
//                 (one tap x 64 input channels, ring of S stages)
//   warp 1        TMEM owner and MMA issuer (one elected thread), M=128,
//                 N=width, K=16 per instruction
//   warps 2..9    epilogue: tcgen05.ld -> (x FP8 scale) + bias -> act ->
//                 BF16 store, zeros on pad rows.  Two warps per TMEM lane
//                 quarter, each taking half of the output channels.  For the
//                 last trunk layer the fused 1x1 head (dot with the head
//                 weights) runs on warps 2..5 over all channels.
// Accumulators are double-buffered in TMEM (2 x N columns), so the epilogue
// of tile i overlaps the MMAs of tile i+1.
//
// Every mbarrier wait is bounded; on a timeout the CTA records an error code,
// stops issuing work, drains what it issued and frees its TMEM.
#include "lg_kernels.h"

#include <cstring>

namespace lg {

using namespace ptx;

constexpr int kTcThreads = 320;
constexpr int kEpiWarps = 8;
// Kernel T: 2 control warps + 16 epilogue warps (4 per TMEM lane quarter).
constexpr int kTcThreadsT = 576;
// Kernel "trunk": + one window-producer warp (18).  19 warps put 5 on one of
// the SM's four sub-partitions (16,384 registers each): at most 96 a thread.
constexpr int kTrunkThreads = 608;
constexpr int kEpiWarpsT = 16;
constexpr uint32_t kWaitLimit = 1u << 26;

struct TcParams {
    int f16;  // operands are FP16 (else BF16)
    const float *bias;
    const float *scale;
    const float *head_w;
    int act;
    int rows;
    int ntiles;
    __nv_bfloat16 *out;
    float *parts;
    size_t part_stride;
    int *err;
};

__device__ __forceinline__ int tap_shift(int kind, int t) {
    if (kind == 0) return (t / 3 - 1) * kL3Pitch + (t % 3 - 1);
    return (t - 2) * kL5Pitch;
}

// ReLU, round to nearest even and pack: lo in bits 0..15, hi in 16..31.
__device__ __forceinline__ uint32_t pack_relu_bf16x2(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}

// The same with FP16 operands.
__device__ __forceinline__ uint32_t pack_relu_f16x2(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.relu.f16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}


// Two fused multiply-adds in one packed FP32 instruction (fma.rn.f32x2,
// sm_100 family): d_i = a_i * b + c, each rounded as fmaf.
__device__ __forceinline__ void ffma2(float &d0, float &d1, float a0, float a1, float b, float c) {
    asm("{\n.reg .b64 ra, rb, rc, rd;\nmov.b64 ra, {%2, %3};\nmov.b64 rb, {%4, %4};\n"
        "mov.b64 rc, {%5, %5};\nfma.rn.f32x2 rd, ra, rb, rc;\nmov.b64 {%0, %1}, rd;\n}"
        : "=f"(d0), "=f"(d1)
        : "f"(a0), "f"(a1), "f"(b), "f"(c));
}

__device__ __forceinline__ float act_apply(float v, int act) {
    if (act == LG_ACT_ELU) return (v > 0.0f) ? v : (expf(v) - 1.0f);
    return fmaxf(v, 0.0f);
}

// Where flat input row q of a layer lands: output row in L3 (-1: none),
// whether it is a board point, and the point index b*361 + y*19 + x.
template <int KIND>
__device__ __forceinline__ void row_target(int q, int rows, int &orow, bool &valid, int &point) {
    orow = -1;
    valid = false;
    point = 0;
    if (q >= rows) return;
    if (KIND == 0) {
        const int b = q / kL3Board, r = q % kL3Board, y = r / kL3Pitch, x = r % kL3Pitch;
        orow = q;
        valid = (x < kBoard && y < kBoard);
        point = b * kPoints + y * kBoard + x;
    } else {
        const int b = q / kL5Board, r = q % kL5Board, y = r / kL5Pitch, x = r % kL5Pitch;
        valid = y < kBoard;
        orow = valid ? b * kL3Board + y * kL3Pitch + x : -1;
        point = b * kPoints + y * kBoard + x;
    }
}

// ===========================================================================
// Kernel A: M = 128 flat rows (positions), N = output channels (any width a
// multiple of 16 up to 256; used for 64-wide nets).  Weight slices stream
// through a ring; the window of rows is the A operand.
// ===========================================================================

template <int N, int HALVES, int KIND>
struct TcCfg {
    static constexpr int NTAPS = KIND == 0 ? 9 : 5;
    static constexpr int WPRE = KIND == 0 ? 24 : 40;
    static constexpr int WROWS = 128 + 2 * WPRE;
    static constexpr int WIN_HALF = WROWS * 128;
    static constexpr int WIN_BYTES = HALVES * WIN_HALF;
    static constexpr int WST_BYTES = N * 128;
    static constexpr int BUDGET = 220 * 1024;
    static constexpr int S_RAW = (BUDGET - 2 * WIN_BYTES) / WST_BYTES;
    static constexpr int S = S_RAW > 8 ? 8 : S_RAW;
    static constexpr int SMEM = 1024 + 2 * WIN_BYTES + S * WST_BYTES;
    static constexpr int TMEM_COLS = 2 * N <= 32 ? 32 : (2 * N <= 64 ? 64 : (2 * N <= 128 ? 128 : 256));
    static_assert(S >= 2, "not enough shared memory for the weight ring");
    static_assert(SMEM <= 227 * 1024, "shared memory budget");
};

template <int N, int HALVES, int KIND, bool HEAD>
__global__ void __launch_bounds__(kTcThreads, 1)
    tc_conv_kernel(const __grid_constant__ CUtensorMap in_map,
                   const __grid_constant__ CUtensorMap w_map, const TcParams p) {
    using C = TcCfg<N, HALVES, KIND>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *win = smem;                       // 2 x WIN_BYTES
    uint8_t *wst = smem + 2 * C::WIN_BYTES;    // S x WST_BYTES

    __shared__ uint64_t win_full[2], win_empty[2], w_full[C::S], w_empty[C::S];
    __shared__ uint64_t acc_full[2], acc_empty[2], mma_done;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    __shared__ float s_bias[N], s_scale[N], s_head[N];

    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(&win_full[i], 1);
            mbar_init(&win_empty[i], 1);
            mbar_init(&acc_full[i], 1);
            mbar_init(&acc_empty[i], kEpiWarps);
        }
        for (int i = 0; i < C::S; ++i) {
            mbar_init(&w_full[i], 1);
            mbar_init(&w_empty[i], 1);
        }
        mbar_init(&mma_done, 1);
        abort_flag = 0;
        fence_mbar_init();
        prefetch_tensormap(&in_map);
        prefetch_tensormap(&w_map);
    }
    for (int i = tid; i < N; i += kTcThreads) {
        s_bias[i] = p.bias[i];
        s_scale[i] = p.scale ? p.scale[i] : 1.0f;
        s_head[i] = HEAD ? p.head_w[i] : 0.0f;
    }
    if (warp == 1) tmem_alloc(&tmem_base, C::TMEM_COLS);
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;

    auto fail = [&](int code) {
        atomicCAS(p.err, 0, code);
        atomicExch(&abort_flag, 1);
    };

    if (warp == 0) {
        // ------------------------------------------------ TMA producer
        if (lane == 0) {
            uint32_t g = 0;
            int local = 0;
            for (int tile = blockIdx.x; tile < p.ntiles && !abort_flag;
                 tile += gridDim.x, ++local) {
                const int wb = local & 1;
                const uint32_t wk = (uint32_t)(local >> 1);
                if (!mbar_wait(&win_empty[wb], (wk & 1) ^ 1, kWaitLimit)) { fail(11); break; }
                mbar_arrive_expect_tx(&win_full[wb], C::WIN_BYTES);
                const int row0 = tile * 128 - C::WPRE;
                for (int h = 0; h < HALVES; ++h)
                    tma_load_2d(win + wb * C::WIN_BYTES + h * C::WIN_HALF, &in_map, &win_full[wb],
                                h * 64, row0);
                for (int t = 0; t < C::NTAPS; ++t)
                    for (int h = 0; h < HALVES; ++h, ++g) {
                        const int s = g % C::S;
                        const uint32_t k = g / C::S;
                        if (!mbar_wait(&w_empty[s], (k & 1) ^ 1, kWaitLimit)) { fail(12); goto done_producer; }
                        mbar_arrive_expect_tx(&w_full[s], C::WST_BYTES);
                        tma_load_2d(wst + s * C::WST_BYTES, &w_map, &w_full[s], 0,
                                    (t * HALVES + h) * N);
                    }
            }
        done_producer:;
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            const uint32_t idesc = idesc_16(128, N, p.f16 != 0);
            uint32_t g = 0;
            int local = 0;
            for (int tile = blockIdx.x; tile < p.ntiles && !abort_flag;
                 tile += gridDim.x, ++local) {
                const int wb = local & 1, acc = local & 1;
                const uint32_t wk = (uint32_t)(local >> 1);
                if (!mbar_wait(&acc_empty[acc], (wk & 1) ^ 1, kWaitLimit)) { fail(21); break; }
                if (!mbar_wait(&win_full[wb], wk & 1, kWaitLimit)) { fail(22); break; }
                tc_fence_after();
                const uint32_t d_tmem = tmem + (uint32_t)(acc * N);
                const uint32_t win_addr = smem_u32(win + wb * C::WIN_BYTES);
                bool first = true;
                for (int t = 0; t < C::NTAPS; ++t) {
                    const uint32_t a_row = (uint32_t)(C::WPRE + tap_shift(KIND, t)) * 128u;
                    for (int h = 0; h < HALVES; ++h, ++g) {
                        const int s = g % C::S;
                        const uint32_t k = g / C::S;
                        if (!mbar_wait(&w_full[s], k & 1, kWaitLimit)) { fail(23); goto done_mma; }
                        tc_fence_after();
                        const uint32_t a_base = win_addr + h * C::WIN_HALF + a_row;
                        const uint32_t b_base = smem_u32(wst + s * C::WST_BYTES);
#pragma unroll
                        for (int kk = 0; kk < 4; ++kk) {
                            mma_bf16(d_tmem, sdesc_sw128(a_base + kk * 32), sdesc_sw128(b_base + kk * 32),
                                     idesc, first ? 0u : 1u);
                            first = false;
                        }
                        mma_commit(&w_empty[s]);
                    }
                }
                mma_commit(&win_empty[wb]);
                mma_commit(&acc_full[acc]);
            }
        done_mma:;
            // every MMA this thread issued has completed before the CTA can
            // free its tensor memory (also after a wait gave up)
            mma_commit(&mma_done);
            mbar_wait(&mma_done, 0, 1u << 20);
        }
    } else {
        // ------------------------------------------------ epilogue
        const int quarter = warp & 3;
        const int chalf = (warp - 2) >> 2;
        const int row = quarter * 32 + lane;
        constexpr int NCOLS = HEAD ? N : N / 2;
        const bool active = HEAD ? (chalf == 0) : true;
        const int cbase = HEAD ? 0 : chalf * (N / 2);
        int local = 0;
        for (int tile = blockIdx.x; tile < p.ntiles && !abort_flag; tile += gridDim.x, ++local) {
            const int acc = local & 1;
            const uint32_t ak = (uint32_t)(local >> 1);
            if (!mbar_wait(&acc_full[acc], ak & 1, kWaitLimit)) { fail(31); break; }
            tc_fence_after();
            if (active) {
                int orow, point;
                bool valid;
                row_target<KIND>(tile * 128 + row, p.rows, orow, valid, point);
                const uint32_t t_row =
                    tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(acc * N + cbase);
                float head_sum = 0.0f;
#pragma unroll 1
                for (int c0 = 0; c0 < NCOLS; c0 += 32) {
                    uint32_t v[32];
                    tmem_ld32(t_row + c0, v);
                    tmem_ld_wait();
                    float f[32];
#pragma unroll
                    for (int i = 0; i < 32; ++i) {
                        const int c = cbase + c0 + i;
                        f[i] = act_apply(fmaf(__uint_as_float(v[i]), s_scale[c], s_bias[c]), p.act);
                    }
                    if (HEAD) {
#pragma unroll
                        for (int i = 0; i < 32; ++i) head_sum = fmaf(f[i], s_head[cbase + c0 + i], head_sum);
                    } else if (orow >= 0) {
                        uint4 pk[4];
                        uint32_t *w32 = reinterpret_cast<uint32_t *>(pk);
#pragma unroll
                        for (int i = 0; i < 16; ++i)
                            w32[i] = valid ? ((uint32_t)round16(f[2 * i], p.f16) |
                                              ((uint32_t)round16(f[2 * i + 1], p.f16) << 16))
                                           : 0u;
                        uint4 *dst = reinterpret_cast<uint4 *>(p.out + (size_t)orow * N + cbase + c0);
#pragma unroll
                        for (int i = 0; i < 4; ++i) dst[i] = pk[i];
                    }
                }
                if (HEAD && valid) p.parts[point] = head_sum;
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[acc]);
        }
    }

    __syncthreads();
    if (abort_flag && tid == 0) {
        // Drain: wait (bounded) for any TMA still in flight into this CTA's
        // shared memory before the CTA exits.
        for (int i = 0; i < 2; ++i) {
            mbar_wait(&win_full[i], 0, 1u << 16);
            mbar_wait(&win_full[i], 1, 1u << 16);
        }
        for (int i = 0; i < C::S; ++i) {
            mbar_wait(&w_full[i], 0, 1u << 16);
            mbar_wait(&w_full[i], 1, 1u << 16);
        }
    }
    __syncthreads();
    tc_fence_after();
    if (warp == 1) tmem_dealloc(tmem, C::TMEM_COLS);
    if (warp == 1) tmem_relinquish();
}

// ===========================================================================
// Kernel T ("transposed"): M = 128 output channels (the weight slice is the
// A operand), N = 256 flat rows (the shifted window is the B operand).  A
// tcgen05 MMA with M=128 needs N=256 to reach the tensor pipe's full rate
// (N <= 128 is bound by the per-instruction time), so 128-wide layers run
// here.  The D tile in TMEM is [channel lane][row column]: the epilogue warp
// for lane quarter q owns channels 32q..32q+31 and stores, per row, one
// 64-byte run of channels.
// ===========================================================================

template <int HALVES, int KIND>
struct TcTCfg {
    static constexpr int NTAPS = KIND == 0 ? 9 : 5;
    static constexpr int TP = 256;  // rows per tile
    static constexpr int WPRE = KIND == 0 ? 24 : 40;
    static constexpr int WROWS = TP + 2 * WPRE;
    static constexpr int SUBROWS = WROWS / 2;   // TMA box rows (<= 256)
    static constexpr int WIN_HALF = WROWS * 128; // one 64-channel half of a window
    static constexpr int NWIN = 3;               // ring of half-windows
    static constexpr int WST_BYTES = 128 * 128;
    // L3 outputs are contiguous rows: the epilogue stages 32 rows x 128
    // channels per row group in shared memory and writes them with one TMA
    // store.  (The first layer's L5 -> L3 row remap stores directly.)
    static constexpr bool STAGED = KIND == 0;
    static constexpr int STG_BYTES = 32 * 256;
    static constexpr int STG_TOTAL = STAGED ? 4 * STG_BYTES : 0;
    static constexpr int BUDGET = 220 * 1024;
    static constexpr int S_RAW = (BUDGET - NWIN * WIN_HALF - STG_TOTAL) / WST_BYTES;
    static constexpr int S = S_RAW > 8 ? 8 : S_RAW;
    static constexpr int SMEM = 1024 + NWIN * WIN_HALF + STG_TOTAL + S * WST_BYTES;
    static_assert(SUBROWS % 8 == 0 && SUBROWS <= 256, "window sub-box");
    static_assert(S >= 3, "not enough shared memory for the weight ring");
    static_assert(SMEM <= 227 * 1024, "shared memory budget");
};

// 32 values per lane -> lane L holds the sum over the warp of value L
// (31 shuffles: each step keeps the half of the values named by one lane bit).
__device__ __forceinline__ float warp_transpose_sum(float (&a)[32], int lane) {
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
        const bool upper = (lane & w) != 0;
#pragma unroll
        for (int i = 0; i < w; ++i) {
            float keep = upper ? a[i + w] : a[i];
            float send = upper ? a[i] : a[i + w];
            a[i] = keep + __shfl_xor_sync(0xffffffffu, send, w);
        }
    }
    return a[0];
}

// Fused 1x1 head: each of a row group's four epilogue warps (one 32-channel
// quarter each) holds its partial sum for the group's 32 rows (lane = row)
// and writes it to its own part, parts[quarter * part_stride + point]; the
// finish kernels add the four parts in quarter order 0..3.  No barrier
// between the warps, so a warp that gave up on a bounded wait can never
// leave the others waiting.
template <int KIND>
__device__ __forceinline__ void head_store(float sum, int quarter, int row, int rows, float *parts,
                                           size_t part_stride) {
    int orow, point;
    bool valid;
    row_target<KIND>(row, rows, orow, valid, point);
    if (valid) parts[(size_t)quarter * part_stride + point] = sum;
}

// Kernel T work split: the rows are cut into 32-row blocks, each CTA takes
// an even contiguous range of blocks and walks it in chunks of up to 256 rows
// (the MMA's N is the chunk's row count), so that no SM runs a whole extra
// 256-row tile at the end of the grid.
__device__ __forceinline__ void cta_row_range(int rows, int &r0, int &r1) {
    const int nblk = (rows + 31) / 32;
    r0 = (int)(((long long)nblk * blockIdx.x) / gridDim.x) * 32;
    r1 = (int)(((long long)nblk * (blockIdx.x + 1)) / gridDim.x) * 32;
}

template <int HALVES, int KIND, bool HEAD>
__global__ void __launch_bounds__(kTcThreadsT, 1)
    tc_convT_kernel(const __grid_constant__ CUtensorMap in_map,
                    const __grid_constant__ CUtensorMap w_map,
                    const __grid_constant__ CUtensorMap out_map, const TcParams p) {
    using C = TcTCfg<HALVES, KIND>;
    constexpr int NO = 128;  // output channels
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *win = smem;                          // NWIN x WIN_HALF
    uint8_t *stg = smem + C::NWIN * C::WIN_HALF;  // 4 x STG_BYTES (staged outputs)
    uint8_t *wst = stg + C::STG_TOTAL;            // S x WST_BYTES

    __shared__ uint64_t win_full[C::NWIN], win_empty[C::NWIN], w_full[C::S], w_empty[C::S];
    __shared__ uint64_t acc_full[2], acc_empty[2], stg_full[4], stg_empty[4], mma_done;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;

    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    if (tid == 0) {
        mbar_init(&mma_done, 1);
        for (int i = 0; i < C::NWIN; ++i) {
            mbar_init(&win_full[i], 1);
            mbar_init(&win_empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&acc_full[i], 1);
            mbar_init(&acc_empty[i], kEpiWarpsT);
        }
        for (int i = 0; i < 4; ++i) {
            mbar_init(&stg_full[i], 4);
            mbar_init(&stg_empty[i], 1);
        }
        for (int i = 0; i < C::S; ++i) {
            mbar_init(&w_full[i], 1);
            mbar_init(&w_empty[i], 1);
        }
        abort_flag = 0;
        fence_mbar_init();
        prefetch_tensormap(&in_map);
        prefetch_tensormap(&w_map);
        if (C::STAGED && !HEAD) prefetch_tensormap(&out_map);
    }
    if (warp == 1) tmem_alloc(&tmem_base, 512);
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;

    auto fail = [&](int code) {
        atomicCAS(p.err, 0, code);
        atomicExch(&abort_flag, 1);
    };

    // K order per tile: channel half h outer, tap t inner, so that half h of
    // the next tile's window loads while half h+1 of this tile computes.
    if (warp == 0) {
        // ------------------------------------------------ TMA producer
        if (lane == 0) {
            uint32_t g = 0, wn = 0;
            int r0, r1;
            cta_row_range(p.rows, r0, r1);
            for (int cs = r0; cs < r1 && !abort_flag; cs += C::TP) {
                const int row0 = cs - C::WPRE;
                for (int h = 0; h < HALVES; ++h, ++wn) {
                    const int ws = wn % C::NWIN;
                    const uint32_t wk = wn / C::NWIN;
                    if (!mbar_wait(&win_empty[ws], (wk & 1) ^ 1, kWaitLimit)) { fail(41); goto done_producer; }
                    mbar_arrive_expect_tx(&win_full[ws], C::WIN_HALF);
                    for (int sb = 0; sb < 2; ++sb)
                        tma_load_2d(win + ws * C::WIN_HALF + sb * C::SUBROWS * 128, &in_map,
                                    &win_full[ws], h * 64, row0 + sb * C::SUBROWS);
                    for (int t = 0; t < C::NTAPS; ++t, ++g) {
                        const int s = g % C::S;
                        const uint32_t k = g / C::S;
                        if (!mbar_wait(&w_empty[s], (k & 1) ^ 1, kWaitLimit)) { fail(42); goto done_producer; }
                        mbar_arrive_expect_tx(&w_full[s], C::WST_BYTES);
                        tma_load_2d(wst + s * C::WST_BYTES, &w_map, &w_full[s], 0,
                                    (t * HALVES + h) * NO);
                    }
                }
            }
        done_producer:;
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            uint32_t g = 0, wn = 0;
            int local = 0;
            int r0, r1;
            cta_row_range(p.rows, r0, r1);
            for (int cs = r0; cs < r1 && !abort_flag; cs += C::TP, ++local) {
                const int nrows = min(C::TP, r1 - cs);
                const uint32_t idesc = idesc_16(128, nrows, p.f16 != 0);
                const int acc = local & 1;
                const uint32_t ak = (uint32_t)(local >> 1);
                if (!mbar_wait(&acc_empty[acc], (ak & 1) ^ 1, kWaitLimit)) { fail(51); break; }
                tc_fence_after();
                const uint32_t d_tmem = tmem + (uint32_t)(acc * C::TP);
                bool first = true;
                for (int h = 0; h < HALVES; ++h, ++wn) {
                    const int ws = wn % C::NWIN;
                    const uint32_t wk = wn / C::NWIN;
                    if (!mbar_wait(&win_full[ws], wk & 1, kWaitLimit)) { fail(52); goto done_mma; }
                    tc_fence_after();
                    const uint32_t win_addr = smem_u32(win + ws * C::WIN_HALF);
                    for (int t = 0; t < C::NTAPS; ++t, ++g) {
                        const int s = g % C::S;
                        const uint32_t k = g / C::S;
                        if (!mbar_wait(&w_full[s], k & 1, kWaitLimit)) { fail(53); goto done_mma; }
                        tc_fence_after();
                        const uint32_t a_base = smem_u32(wst + s * C::WST_BYTES);
                        const uint32_t b_base =
                            win_addr + (uint32_t)(C::WPRE + tap_shift(KIND, t)) * 128u;
#pragma unroll
                        for (int kk = 0; kk < 4; ++kk) {
                            mma_bf16(d_tmem, sdesc_sw128(a_base + kk * 32), sdesc_sw128(b_base + kk * 32),
                                     idesc, first ? 0u : 1u);
                            first = false;
                        }
                        mma_commit(&w_empty[s]);
                    }
                    mma_commit(&win_empty[ws]);
                }
                mma_commit(&acc_full[acc]);
            }
        done_mma:;
            mma_commit(&mma_done);
            mbar_wait(&mma_done, 0, 1u << 20);
        }
    } else {
        // ------------------------------------------------ epilogue
        const int quarter = warp & 3;
        const int rq = (warp - 2) >> 2;          // rows [rq*64, +64) of the tile
        const int o = quarter * 32 + lane;       // this lane's output channel
        const float bias = __ldg(p.bias + o);
        const float scale = p.scale ? __ldg(p.scale + o) : 1.0f;
        const float hw = HEAD ? __ldg(p.head_w + o) : 0.0f;
        int local = 0;
        uint32_t uses = 0;  // staging buffer uses of this row group (same for its 4 warps)
        int r0, r1;
        cta_row_range(p.rows, r0, r1);
        for (int cs = r0; cs < r1 && !abort_flag; cs += C::TP, ++local) {
            const int nrows = min(C::TP, r1 - cs);
            const int nhalf = max(0, min(2, (nrows - rq * 64) / 32));  // 32-row halves of this group
            const int acc = local & 1;
            const uint32_t ak = (uint32_t)(local >> 1);
            if (!mbar_wait(&acc_full[acc], ak & 1, kWaitLimit)) { fail(61); break; }
            tc_fence_after();
            const uint32_t t_base = tmem + ((uint32_t)(quarter * 32) << 16) +
                                    (uint32_t)(acc * C::TP + rq * 64);
            const int q_base = cs + rq * 64;
            // (columns past the chunk are read but unused: the accumulator
            // holds 256 columns whatever the chunk's N)
            uint32_t v[2][32];
            tmem_ld32(t_base, v[0]);
            tmem_ld32(t_base + 32, v[1]);
            tmem_ld_wait();
            tc_fence_before();
            __syncwarp();
            // TMEM is read: release the accumulator before the stores.
            if (lane == 0) mbar_arrive(&acc_empty[acc]);
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                if (c >= nhalf) break;
                float f[32];
#pragma unroll
                for (int j = 0; j < 32; ++j) f[j] = act_apply(fmaf(__uint_as_float(v[c][j]), scale, bias), p.act);
                if (HEAD) {
#pragma unroll
                    for (int j = 0; j < 32; ++j) f[j] *= hw;
                    head_store<KIND>(warp_transpose_sum(f, lane), quarter, q_base + c * 32 + lane, p.rows, p.parts,
                                     p.part_stride);
                } else if (C::STAGED) {
                    // Rows q_base + c*32 .. +31 -> staging buffer of this row
                    // group as [32 rows][128 channels] BF16 (pad rows 0), then
                    // one TMA store by the group's quarter-0 warp.
                    const uint32_t use = uses++;
                    uint8_t *buf = stg + rq * C::STG_BYTES;
                    if (!mbar_wait(&stg_empty[rq], (use & 1) ^ 1, kWaitLimit)) { fail(62); break; }
                    const int row_lane = q_base + c * 32 + lane;
                    const int rl = row_lane % kL3Board;
                    const bool valid_lane = (rl % kL3Pitch) < kBoard && (rl / kL3Pitch) < kBoard;
                    const unsigned vmask = __ballot_sync(0xffffffffu, valid_lane);
                    uint16_t *col = reinterpret_cast<uint16_t *>(buf) + o;
#pragma unroll
                    for (int j = 0; j < 32; ++j) col[j * 128] = round16(((vmask >> j) & 1u) ? f[j] : 0.0f, p.f16);
                    fence_proxy_async();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&stg_full[rq]);
                    if (quarter == 0 && lane == 0) {
                        if (!mbar_wait(&stg_full[rq], use & 1, kWaitLimit)) {
                            fail(63);
                        } else {
                            tma_store_2d(&out_map, buf, 0, q_base + c * 32);
                            bulk_commit();
                            bulk_wait_read0();
                        }
                        mbar_arrive(&stg_empty[rq]);
                    }
                    __syncwarp();
                } else {
                    // Lane j works out where row (c*32 + j) goes once; the warp
                    // then walks the 32 rows with that code broadcast:
                    // -1 = no output, >= 0 = board point row, <= -2 = pad
                    // row -(code + 2) (written as zero).
                    int orow, point;
                    bool valid;
                    row_target<KIND>(q_base + c * 32 + lane, p.rows, orow, valid, point);
                    const int code = orow < 0 ? -1 : (valid ? orow : -(orow + 2));
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        const int cj = __shfl_sync(0xffffffffu, code, j);
                        if (cj != -1) {
                            const int r = cj >= 0 ? cj : -(cj + 2);
                            reinterpret_cast<uint16_t *>(p.out)[(size_t)r * NO + o] = round16(cj >= 0 ? f[j] : 0.0f, p.f16);
                        }
                    }
                }
            }
        }
    }

    if (C::STAGED && !HEAD && warp >= 2 && (warp & 3) == 0 && lane == 0) bulk_wait0();
    __syncthreads();
    if (abort_flag && tid == 0) {
        for (int i = 0; i < C::NWIN; ++i) {
            mbar_wait(&win_full[i], 0, 1u << 16);
            mbar_wait(&win_full[i], 1, 1u << 16);
        }
        for (int i = 0; i < C::S; ++i) {
            mbar_wait(&w_full[i], 0, 1u << 16);
            mbar_wait(&w_full[i], 1, 1u << 16);
        }
    }
    __syncthreads();
    tc_fence_after();
    if (warp == 1) tmem_dealloc(tmem, 512);
    if (warp == 1) tmem_relinquish();
}

// ===========================================================================
// Kernel "trunk": every 3x3 128->128 layer of a net in one persistent
// launch, scheduled as work items (layer l, chunk j) of 256 rows (224 for
// the fused 5x5 first layer's items).  The
// producer of each CTA claims items from a global counter in (layer, chunk)
// order and runs kernel T's pipeline over each (its windows, weight stages,
// MMAs, epilogue), ping-ponging between two L3 buffers (layer l reads A when
// l is even, B when odd).  Item (l, j) reads rows [256j - 24, 256j + 280) of
// layer l-1's output, written by items (l-1, j-1 .. j+1), and overwrites rows
// that only those items read for layer l-1: so it starts once flags[j-1 ..
// j+1] >= l.  flags[j] = number of layers whose chunk-j rows are stored
// (published with release after the item's TMA stores completed; the
// producer polls with acquire, bounded).  Items are claimed in order, so an
// item's dependencies were claimed earlier by CTAs that are running: there
// is no layer-wide barrier, faster SMs take more items, and every item but a
// layer's last runs at N = 256.  The last layer can carry the fused 1x1 head.
// ===========================================================================

struct TrunkParams {
    const float *bias;    // [nl][128], the 3x3 layers
    const float *scale;   // [nl][128] or null
    const float *bias0;   // [128]: the fused 5x5 first layer (rows5 > 0)
    const float *scale0;  // [128] or null
    const float *head_w;  // [128] (HEAD)
    __nv_bfloat16 *out0;  // the first layer's output rows (buffer A)
    int act;
    int rows;             // L3 rows, B * 400
    int rows5;            // L5 rows of the fused first layer, B * 399; 0 = none
    int nl;               // 3x3 layers
    float *parts;
    size_t part_stride;
    int *flags;           // [n3] chunk flags, the item counter, [n5] first-layer chunk flags, the
                          // exit counter: zero at entry, and the last CTA to leave zeroes them
    int *err;
    uint32_t wait_limit;  // polls of one mbarrier wait before it gives up
    uint32_t poll_limit;  // polls of one dependency flag before it gives up
    int stall_item;       // test hook: this item waits for a flag nothing sets (-1: none)
    const int *count;     // device-side batch size (boards), or null: all of rows
    int count_base;       // boards before this launch's first
};

constexpr uint32_t kFlagPolls = 1u << 22;  // x ~64 ns sleep: bounded at ~0.3 s
constexpr int kItemRing = 4;               // item descriptors in flight per CTA

// The trunk's barriers and item ring, kept after its buffers in the dynamic
// shared memory (the kernel has no static shared memory, so the buffers can
// use all but the alignment slack of the 227 KB a CTA may have).
template <int NWIN, int S>
struct TrunkCtl {
    uint64_t win_full[NWIN], win_empty[NWIN], w_full[S], w_empty[S];
    uint64_t acc_full[2], acc_empty[2], stg_full[4], stg_empty[4], item_done[4], mma_done;
    uint64_t item_full[kItemRing], item_empty[kItemRing];
    int item_id[kItemRing];
    uint32_t tmem_base;
    int abort_flag;
    int last_out;
};

// Shared memory of kernel "trunk": three half-window slots, four staging
// tiles, five weight stages, the control block.  A 3x3 item covers 256 rows
// (window 256 + 2 x 24); a first-layer item covers 224 rows so that its
// window (5 taps of pitch 19: 224 + 2 x 40) fits the same slot: the fifth
// weight stage lives in the bytes a taller slot would take.  The buffers
// start at the first 1024-byte boundary of the dynamic region (the 128-byte
// swizzle's alignment); PAD is the slack left for that.
struct TrunkCfg {
    using C0 = TcTCfg<2, 0>;
    using C1 = TcTCfg<2, 1>;
    static constexpr int TP = 256;
    static constexpr int TP5 = 224;
    static constexpr int WIN5_ROWS = TP5 + 2 * C1::WPRE;
    static constexpr int SUB5 = WIN5_ROWS / 2;  // TMA box rows of a first-layer half-window
    static constexpr int WIN5_HALF = WIN5_ROWS * 128;
    static constexpr int NWIN = 3;
    static constexpr int WIN_SLOT = WIN5_HALF > C0::WIN_HALF ? WIN5_HALF : C0::WIN_HALF;
    static constexpr int S = 5;
    static constexpr int WST_BYTES = C0::WST_BYTES;
    static constexpr int STG_BYTES = C0::STG_BYTES;
    static constexpr int STG_TOTAL = 4 * STG_BYTES;
    using Ctl = TrunkCtl<NWIN, S>;
    static constexpr int CTL_OFF = NWIN * WIN_SLOT + STG_TOTAL + S * WST_BYTES;
    static constexpr int SMEM = 227 * 1024;
    static constexpr int PAD = SMEM - CTL_OFF - (int)sizeof(Ctl);
    static_assert(C0::TP == TP && TP5 % 16 == 0 && TP5 <= TP, "item rows");
    static_assert(WIN_SLOT % 1024 == 0 && (C0::SUBROWS * 128) % 1024 == 0 && (SUB5 * 128) % 1024 == 0,
                  "window boxes keep the 1024-byte swizzle alignment");
    static_assert(CTL_OFF % 8 == 0 && PAD >= 0, "shared memory budget");
};

// The MMAs of one 64-channel half of an item: NTAPS weight stages (one per
// tap, 4 K steps of 16 each) against the window in the slot whose descriptor
// is b_desc; stage g of the ring is slot g % NS.  Descriptor start addresses
// advance by (bytes >> 4): tap rows of 128 bytes, K steps of 32 bytes.
// Returns false if a weight stage did not arrive within the wait limit.
template <int KIND, int NTAPS, int WPRE, int NS>
__device__ __forceinline__ bool issue_taps(uint32_t d_tmem, uint64_t a_desc0, uint64_t b_desc, uint32_t idesc,
                                           bool first_half, uint32_t &g, uint64_t *w_full, uint64_t *w_empty,
                                           uint32_t wl) {
    constexpr int kStage16 = TcTCfg<2, 0>::WST_BYTES >> 4;
#pragma unroll
    for (int t = 0; t < NTAPS; ++t, ++g) {
        const int s = (int)(g % NS);
        if (!mbar_wait(&w_full[s], (g / NS) & 1, wl)) return false;
        tc_fence_after();
        const uint64_t a = a_desc0 + (uint64_t)(s * kStage16);
        const uint64_t b = b_desc + (uint64_t)((WPRE + (KIND == 0 ? (t / 3 - 1) * kL3Pitch + (t % 3 - 1)
                                                                  : (t - 2) * kL5Pitch)) * 8);
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
            mma_bf16(d_tmem, a + 2 * kk, b + 2 * kk, idesc, (first_half && t == 0 && kk == 0) ? 0u : 1u);
        mma_commit(&w_empty[s]);
    }
    return true;
}

__device__ __forceinline__ bool poll_flag(const int *f, int want, uint32_t limit) {
    uint32_t n = 0;
    while (ld_acquire_gpu(f) < want && ++n < limit) __nanosleep(64);
    return n < limit;
}

template <bool HEAD, bool F16>
__global__ void __maxnreg__(96)
    tc_trunk_kernel(const __grid_constant__ CUtensorMap in_a, const __grid_constant__ CUtensorMap in_b,
                    const __grid_constant__ CUtensorMap out_a, const __grid_constant__ CUtensorMap out_b,
                    const __grid_constant__ CUtensorMap w_map, const __grid_constant__ CUtensorMap in5,
                    const __grid_constant__ CUtensorMap w0_map, const __grid_constant__ CUtensorMap out_a_sw,
                    const __grid_constant__ CUtensorMap out_b_sw, const TrunkParams p) {
    using C = TrunkCfg;
    using C0 = TrunkCfg::C0;
    using C1 = TrunkCfg::C1;
    constexpr int HALVES = 2, NO = 128;
    extern __shared__ uint8_t smem_raw[];
    // The buffers need a 1024-byte aligned base; with no static shared
    // memory the dynamic region starts aligned, and PAD bytes of slack cover
    // a base that does not.  A launch without room reports code 69.
    const uint32_t mis = (1024u - (smem_u32(smem_raw) & 1023u)) & 1023u;
    if (mis > (uint32_t)C::PAD) {
        if (threadIdx.x == 0) atomicCAS(p.err, 0, 69);
        return;
    }
    uint8_t *smem = smem_raw + mis;
    uint8_t *win = smem;
    uint8_t *stg = smem + C::NWIN * C::WIN_SLOT;
    uint8_t *wst = stg + C::STG_TOTAL;
    TrunkCfg::Ctl &ctl = *reinterpret_cast<TrunkCfg::Ctl *>(smem + C::CTL_OFF);
    uint64_t *const win_full = ctl.win_full, *const win_empty = ctl.win_empty;
    uint64_t *const w_full = ctl.w_full, *const w_empty = ctl.w_empty;
    // item_done: a ring of 4 (an epilogue warp can be up to two items ahead
    // of the slowest: starting item x needs every warp to have read item
    // x-2's accumulator, hence to have arrived for item x-3)
    uint64_t *const acc_full = ctl.acc_full, *const acc_empty = ctl.acc_empty;
    uint64_t *const stg_full = ctl.stg_full, *const stg_empty = ctl.stg_empty;
    uint64_t *const item_done = ctl.item_done, &mma_done = ctl.mma_done;
    uint64_t *const item_full = ctl.item_full, *const item_empty = ctl.item_empty;
    int *const item_id = ctl.item_id;
    uint32_t &tmem_base = ctl.tmem_base;
    int &abort_flag = ctl.abort_flag;

    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
#define WAIT_LIM (p.wait_limit)  // mbarrier waits (try_wait polls): read from the parameter bank at each use
    // rows / rows5: the rows this launch computes (with a device-side count,
    // the first *count - count_base boards); the flag layout follows the
    // buffers' extent p.rows
    int rows = p.rows, rows5 = p.rows5;
    if (p.count) {
        grid_dep_wait();  // the count was written by an earlier kernel
        const int nb = min(p.rows / kL3Board, max(0, *p.count - p.count_base));
        rows = nb * kL3Board;
        rows5 = p.rows5 > 0 ? nb * kL5Board : 0;
    }
    const int n3L = (p.rows + C::TP - 1) / C::TP;
    const int n3 = (rows + C::TP - 1) / C::TP;
    const int n5 = rows5 > 0 ? (rows5 + C::TP5 - 1) / C::TP5 : 0;
    const int first = p.rows5 > 0 ? 1 : 0;
    const int nitems = n5 + p.nl * n3;
    int *const flags0 = p.flags + n3L + 1;
    // item -> (layer l, chunk j); layer 0 is the first layer when fused
    auto decode = [&](int it, int &l, int &j) {
        if (it < n5) {
            l = 0;
            j = it;
        } else {
            const int r = it - n5;
            l = first + r / n3;
            j = r - (r / n3) * n3;
        }
    };
    if (tid == 0) {
        for (int i = 0; i < C::NWIN; ++i) {
            mbar_init(&win_full[i], 1);
            mbar_init(&win_empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&acc_full[i], 1);
            mbar_init(&acc_empty[i], kEpiWarpsT);
        }
        for (int i = 0; i < 4; ++i) {
            mbar_init(&stg_full[i], 4);
            mbar_init(&stg_empty[i], 1);
        }
        for (int i = 0; i < C::S; ++i) {
            mbar_init(&w_full[i], 1);
            mbar_init(&w_empty[i], 1);
        }
        for (int i = 0; i < kItemRing; ++i) {
            mbar_init(&item_full[i], 1);
            mbar_init(&item_empty[i], 2 + kEpiWarpsT);  // weight producer, MMA issuer, epilogue warps
        }
        for (int i = 0; i < 4; ++i) mbar_init(&item_done[i], kEpiWarpsT);
        mbar_init(&mma_done, 1);
        abort_flag = 0;
        fence_mbar_init();
        prefetch_tensormap(&in_a);
        prefetch_tensormap(&in_b);
        prefetch_tensormap(&out_a);
        prefetch_tensormap(&out_b);
        prefetch_tensormap(&out_a_sw);
        prefetch_tensormap(&out_b_sw);
        prefetch_tensormap(&w_map);
        if (first) {
            prefetch_tensormap(&in5);
            prefetch_tensormap(&w0_map);
        }
    }
    if (warp == 1) tmem_alloc(&tmem_base, 512);
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    // Launched as a programmatic dependent of the previous kernel, the
    // prologue above (barriers, TMEM, tensor-map prefetch: no global memory)
    // overlapped it; everything below may read what it wrote.  The next
    // kernel may then be scheduled as this one's CTAs leave.
    grid_dep_wait();
    grid_dep_launch();

    auto fail = [&](int code) {
        atomicCAS(p.err, 0, code);
        atomicExch(&abort_flag, 1);
    };

    if (warp == kEpiWarpsT + 2) {
        // ------------------------------------------------ item claims + windows
        if (lane == 0) {
            uint32_t wn = 0;
            for (int q = 0;; ++q) {
                const int slot = q % kItemRing;
                const uint32_t qk = (uint32_t)(q / kItemRing);
                // Claim only once the item ring and the next window slot are
                // free, so that a claimed item is worked on at once.
                bool ok = mbar_wait(&item_empty[slot], (qk & 1) ^ 1, WAIT_LIM);
                const int ws0 = wn % C::NWIN;
                ok = ok && mbar_wait(&win_empty[ws0], ((wn / C::NWIN) & 1) ^ 1, WAIT_LIM);
                int it = -1;
                if (ok && !abort_flag) {
                    it = atomicAdd(p.flags + n3L, 1);
                    if (it >= nitems) it = -1;
                } else if (!ok) {
                    fail(72);
                }
                item_id[slot] = it;
                mbar_arrive(&item_full[slot]);  // releases item_id[slot]
                if (it < 0) break;
                int l, j;
                decode(it, l, j);
                const bool fl = first && l == 0;
                const int k = l - first;  // 3x3 layer index
                if (!fl && k == 0 && first) {
                    // the first layer's chunks whose L5 rows feed L3 rows
                    // [256j - 24, 256j + 280): an L5 row is the L3 row minus
                    // (board + y), board + y <= rows / 400 + 19
                    const int lo3 = max(0, j * C::TP - C0::WPRE);
                    const int hi3 = min(rows, j * C::TP + C::TP + C0::WPRE);
                    const int lo5 = max(0, lo3 - (hi3 - 1) / kL3Board - kBoard);
                    const int hi5 = min(rows5 - 1, hi3 - 1);
                    for (int jj = lo5 / C::TP5; jj <= hi5 / C::TP5; ++jj)
                        if (!poll_flag(flags0 + jj, 1, p.poll_limit)) {
                            fail(71);
                            goto done_windows;
                        }
                    fence_proxy_async_global();
                } else if (!fl && k > 0) {
                    // layer k-1 of chunks j-1 .. j+1 is stored
                    const int lo = max(0, j - 1), hi = min(n3 - 1, j + 1);
                    // (test hook: the stalled item waits for a layer count
                    // no item ever publishes)
                    const int want = it == p.stall_item ? (1 << 30) : k;
                    for (int jj = lo; jj <= hi; ++jj)
                        if (!poll_flag(p.flags + jj, want, p.poll_limit)) {
                            fail(71);
                            goto done_windows;
                        }
                    fence_proxy_async_global();
                }
                const CUtensorMap *im = fl ? &in5 : ((k & 1) ? &in_b : &in_a);
                const int sub = fl ? C::SUB5 : C0::SUBROWS;
                const uint32_t bytes = fl ? C::WIN5_HALF : C0::WIN_HALF;
                const int row0 = fl ? j * C::TP5 - C1::WPRE : j * C::TP - C0::WPRE;
                for (int h = 0; h < HALVES; ++h, ++wn) {
                    const int ws = wn % C::NWIN;
                    const uint32_t wk = wn / C::NWIN;
                    // (the first half's slot was waited for before the claim)
                    if (h > 0 && !mbar_wait(&win_empty[ws], (wk & 1) ^ 1, WAIT_LIM)) { fail(73); goto done_windows; }
                    mbar_arrive_expect_tx(&win_full[ws], bytes);
                    for (int sb = 0; sb < 2; ++sb)
                        tma_load_2d(win + ws * C::WIN_SLOT + sb * sub * 128, im, &win_full[ws], h * 64,
                                    row0 + sb * sub);
                }
            }
        done_windows:;
        }
    } else if (warp == 0) {
        // ------------------------------------------------ weight stages
        if (lane == 0) {
            uint32_t g = 0;
            for (int q = 0;; ++q) {
                const int slot = q % kItemRing;
                if (!mbar_wait(&item_full[slot], (uint32_t)(q / kItemRing) & 1, WAIT_LIM)) { fail(70); break; }
                const int it = item_id[slot];
                mbar_arrive(&item_empty[slot]);
                if (it < 0) break;
                int l, j;
                decode(it, l, j);
                const bool fl = first && l == 0;
                const int ntaps = fl ? C1::NTAPS : C0::NTAPS;
                const CUtensorMap *wm = fl ? &w0_map : &w_map;
                const int wl = fl ? 0 : l - first;
                for (int h = 0; h < HALVES; ++h) {
                    for (int t = 0; t < ntaps; ++t, ++g) {
                        const int s = g % C::S;
                        const uint32_t k = g / C::S;
                        if (!mbar_wait(&w_empty[s], (k & 1) ^ 1, WAIT_LIM)) { fail(74); goto done_weights; }
                        mbar_arrive_expect_tx(&w_full[s], C::WST_BYTES);
                        tma_load_2d(wst + s * C::WST_BYTES, wm, &w_full[s], 0, ((wl * ntaps + t) * HALVES + h) * NO);
                    }
                }
            }
        done_weights:;
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer
        // One thread keeps the tensor pipe fed: every descriptor is a base
        // computed once plus compile-time offsets (tap rows, K steps), and the
        // tap and K loops are unrolled per item kind, so issuing an MMA costs
        // a 64-bit add per operand (an MMA of N = 256 lasts ~128 cycles).
        if (lane == 0) {
            const uint64_t a_desc0 = sdesc_sw128(smem_u32(wst));
            const uint64_t b_desc0 = sdesc_sw128(smem_u32(win));
            uint32_t g = 0, wn = 0;
            for (int q = 0;; ++q) {
                const int slot = q % kItemRing;
                if (!mbar_wait(&item_full[slot], (uint32_t)(q / kItemRing) & 1, WAIT_LIM)) { fail(75); break; }
                const int it = item_id[slot];
                mbar_arrive(&item_empty[slot]);
                if (it < 0) break;
                int l, j;
                decode(it, l, j);
                const bool fl = first && l == 0;
                // N: the item's rows, rounded up to the MMA's multiple of 16
                // (rows past the tensor are zero-filled and not stored)
                const int nrows = fl ? min(C::TP5, (rows5 - j * C::TP5 + 15) / 16 * 16) : min(C::TP, rows - j * C::TP);
                const uint32_t idesc = idesc_16(128, nrows, F16);
                const int acc = q & 1;
                const uint32_t ak = (uint32_t)(q >> 1);
                if (!mbar_wait(&acc_empty[acc], (ak & 1) ^ 1, WAIT_LIM)) { fail(76); break; }
                tc_fence_after();
                const uint32_t d_tmem = tmem + (uint32_t)(acc * C::TP);
                bool ok = true;
#pragma unroll
                for (int h = 0; h < HALVES && ok; ++h, ++wn) {
                    const int ws = wn % C::NWIN;
                    const uint32_t wk = wn / C::NWIN;
                    if (!mbar_wait(&win_full[ws], wk & 1, WAIT_LIM)) { fail(77); ok = false; break; }
                    tc_fence_after();
                    const uint64_t b_desc = b_desc0 + (uint64_t)(ws * (C::WIN_SLOT >> 4));
                    ok = fl ? issue_taps<1, C1::NTAPS, C1::WPRE, C::S>(d_tmem, a_desc0, b_desc, idesc, h == 0, g, w_full,
                                                                 w_empty, WAIT_LIM)
                            : issue_taps<0, C0::NTAPS, C0::WPRE, C::S>(d_tmem, a_desc0, b_desc, idesc, h == 0, g, w_full,
                                                                 w_empty, WAIT_LIM);
                    if (!ok) { fail(78); break; }
                    mma_commit(&win_empty[ws]);
                }
                if (!ok) break;
                mma_commit(&acc_full[acc]);
            }
            // every MMA this thread issued has completed before the CTA can
            // free its tensor memory (also after a wait gave up)
            mma_commit(&mma_done);
            mbar_wait(&mma_done, 0, 1u << 20);
        }
    } else {
        // ------------------------------------------------ epilogue
        const int quarter = warp & 3;
        const int rq = (warp - 2) >> 2;
        const int o = quarter * 32 + lane;
        const float hw = HEAD ? __ldg(p.head_w + o) : 0.0f;
        uint32_t uses = 0, done_n = 0;
        for (int q = 0;; ++q) {
            const int slot = q % kItemRing;
            if (!mbar_wait(&item_full[slot], (uint32_t)(q / kItemRing) & 1, WAIT_LIM)) { fail(79); break; }
            const int it = item_id[slot];
            __syncwarp();
            if (lane == 0) mbar_arrive(&item_empty[slot]);
            if (it < 0) break;
            int l, j;
            decode(it, l, j);
            const bool fl = first && l == 0;
            const int k = l - first;
            const int cs = j * (fl ? C::TP5 : C::TP);
            const float bias = fl ? __ldg(p.bias0 + o) : __ldg(p.bias + k * NO + o);
            const float scale = fl ? (p.scale0 ? __ldg(p.scale0 + o) : 1.0f)
                                   : (p.scale ? __ldg(p.scale + k * NO + o) : 1.0f);
            const bool head_layer = HEAD && !fl && k == p.nl - 1;
            const CUtensorMap *om = (k & 1) ? &out_a : &out_b;
            const int rows_l = fl ? rows5 : rows;
            const int nrows = min(fl ? C::TP5 : C::TP, rows_l - cs);
            const int nhalf = max(0, min(2, (nrows - rq * 64 + 31) / 32));
            const int acc = q & 1;
            const uint32_t ak = (uint32_t)(q >> 1);
            if (!mbar_wait(&acc_full[acc], ak & 1, WAIT_LIM)) { fail(80); break; }
            tc_fence_after();
            const uint32_t t_base = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(acc * C::TP + rq * 64);
            const int q_base = cs + rq * 64;
            bool bad = false;
            // 3x3 ReLU items take the fragment path: TMEM read as the MMA
            // accumulator fragments (16x256b: thread t holds channels
            // t/4 + {0, 8, 16, 24} of its quarter for row pairs), packed and
            // written with stmatrix.trans into a 128-byte-swizzled staging
            // tile (two 64-channel halves), stored by two TMA boxes.  Head,
            // first-layer and ELU items keep the 32x32b path below.
            if (!fl && !head_layer && p.act == LG_ACT_RELU) {
                const float *bl = p.bias + k * NO, *sl = p.scale ? p.scale + k * NO : nullptr;
                const int cq = quarter * 32 + (lane >> 2);
                float fb[4], fs[4];
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    fb[m] = __ldg(bl + cq + 8 * m);
                    fs[m] = sl ? __ldg(sl + cq + 8 * m) : 1.0f;
                }
                const CUtensorMap *om_sw = (k & 1) ? &out_a_sw : &out_b_sw;
                const int hh = quarter >> 1;
                const uint32_t stg_half = smem_u32(stg + rq * C::STG_BYTES + hh * (C::STG_BYTES / 2));
                const uint32_t st_addr =
                    stg_half + (lane & 7) * 128 + (((((quarter & 1) * 4) + (lane >> 3)) ^ (lane & 7)) * 16);
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    uint32_t r0[16], r1[16];
                    tmem_ld16x256_x4(t_base + 32 * c, r0);
                    tmem_ld16x256_x4(t_base + (16u << 16) + 32 * c, r1);
                    tmem_ld_wait();
                    if (c == 1) {
                        tc_fence_before();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&acc_empty[acc]);
                    }
                    if (c >= nhalf || bad) continue;
                    const uint32_t use = uses++;
                    if (!mbar_wait(&stg_empty[rq], (use & 1) ^ 1, WAIT_LIM)) {
                        fail(81);
                        bad = true;
                        continue;
                    }
                    const int rl = (q_base + c * 32 + lane) % kL3Board;
                    const unsigned vmask = __ballot_sync(0xffffffffu, (rl % kL3Pitch) < kBoard && (rl / kL3Pitch) < kBoard);
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        uint32_t w[4];
#pragma unroll
                        for (int m = 0; m < 4; ++m) {
                            const uint32_t *rr = (m < 2) ? r0 : r1;
                            float a0, a1;
                            ffma2(a0, a1, __uint_as_float(rr[4 * i + 2 * (m & 1)]),
                                  __uint_as_float(rr[4 * i + 2 * (m & 1) + 1]), fs[m], fb[m]);
                            w[m] = F16 ? pack_relu_f16x2(a0, a1) : pack_relu_bf16x2(a0, a1);
                        }
                        stmatrix_x4_trans(st_addr + i * 1024, w[0], w[1], w[2], w[3]);
                    }
                    __syncwarp();
                    // pad rows (x = 19, y = 19) as zeros: lane L clears row
                    // 8g + L/4, chunk L%4 of this quarter's 64 bytes
#pragma unroll
                    for (int g = 0; g < 4; ++g) {
                        const int row = 8 * g + (lane >> 2);
                        if (!((vmask >> row) & 1u)) {
                            const uint32_t za = stg_half + row * 128 + ((((quarter & 1) * 4 + (lane & 3)) ^ (row & 7)) * 16);
                            asm volatile("st.shared.v4.b32 [%0], {%1,%1,%1,%1};" ::"r"(za), "r"(0u) : "memory");
                        }
                    }
                    fence_proxy_async();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&stg_full[rq]);
                    if (quarter == 0 && lane == 0) {
                        if (!mbar_wait(&stg_full[rq], use & 1, WAIT_LIM)) {
                            fail(82);
                        } else {
                            uint8_t *buf = stg + rq * C::STG_BYTES;
                            tma_store_2d(om_sw, buf, 0, q_base + c * 32);
                            tma_store_2d(om_sw, buf + C::STG_BYTES / 2, 64, q_base + c * 32);
                            bulk_commit();
                            bulk_wait_read0();
                        }
                        mbar_arrive(&stg_empty[rq]);
                    }
                    __syncwarp();
                }
            }
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                if (!fl && !head_layer && p.act == LG_ACT_RELU) break;
                // One 32-row half at a time (32 registers); the accumulator is
                // released after the second half's load, which the MMA issuer
                // needs again only one item later.
                uint32_t v[32];
                tmem_ld32(t_base + 32 * c, v);
                tmem_ld_wait();
                if (c == 1) {
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&acc_empty[acc]);
                }
                if (c >= nhalf || bad) continue;
                if (head_layer) {
                    float f[32];
#pragma unroll
                    for (int jj = 0; jj < 32; ++jj)
                        f[jj] = act_apply(fmaf(__uint_as_float(v[jj]), scale, bias), p.act) * hw;
                    head_store<0>(warp_transpose_sum(f, lane), quarter, q_base + c * 32 + lane, rows, p.parts,
                                  p.part_stride);
                } else {
                    const uint32_t use = uses++;
                    uint8_t *buf = stg + rq * C::STG_BYTES;
                    if (!mbar_wait(&stg_empty[rq], (use & 1) ^ 1, WAIT_LIM)) {
                        fail(81);
                        bad = true;
                        continue;
                    }
                    const int row_lane = q_base + c * 32 + lane;
                    // 3x3 items: L3 rows, pad rows written as zeros.  First-
                    // layer items: L5 rows; lane's L3 row (-1: pad row y =
                    // 19, 20 or past the last board, not stored).
                    int orow = -1;
                    bool valid_lane;
                    if (fl) {
                        int point;
                        row_target<1>(row_lane, rows5, orow, valid_lane, point);
                    } else {
                        const int rl = row_lane % kL3Board;
                        valid_lane = (rl % kL3Pitch) < kBoard && (rl / kL3Pitch) < kBoard;
                    }
                    const unsigned vmask = __ballot_sync(0xffffffffu, valid_lane);
                    // This warp shares its SM sub-partition's issue slots with
                    // the MMA-issuing thread (a warp reads only the TMEM lane
                    // quarter of its sub-partition), so the loop is lean:
                    // per two rows one packed scale + bias (fma.rn.f32x2), one
                    // ReLU + round + pack (cvt.rn.relu.bf16x2), two 16-bit
                    // stores; pad rows are zeroed afterwards.
                    uint16_t *col = reinterpret_cast<uint16_t *>(buf) + o;
                    if (p.act == LG_ACT_RELU) {
#pragma unroll
                        for (int jj = 0; jj < 32; jj += 2) {
                            float a0, a1;
                            ffma2(a0, a1, __uint_as_float(v[jj]), __uint_as_float(v[jj + 1]), scale, bias);
                            const uint32_t w = F16 ? pack_relu_f16x2(a0, a1) : pack_relu_bf16x2(a0, a1);
                            col[jj * 128] = (uint16_t)w;
                            col[(jj + 1) * 128] = (uint16_t)(w >> 16);
                        }
                    } else {
#pragma unroll
                        for (int jj = 0; jj < 32; ++jj)
                            col[jj * 128] = round16(act_apply(fmaf(__uint_as_float(v[jj]), scale, bias), p.act), F16);
                    }
                    for (unsigned pad = ~vmask; pad; pad &= pad - 1) col[(__ffs(pad) - 1) * 128] = 0;
                    fence_proxy_async();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&stg_full[rq]);
                    if (quarter == 0) {
                        // every lane of the warp holds its row's target; lane 0 stores
                        const bool ok = lane != 0 || mbar_wait(&stg_full[rq], use & 1, WAIT_LIM);
                        if (!ok) fail(82);
                        if (!fl) {
                            if (lane == 0 && ok) tma_store_2d(om, buf, 0, q_base + c * 32);
                        } else {
                            // runs of rows whose L3 rows are consecutive: one
                            // plain bulk copy each (at most 3 per 32 rows)
                            const int prev = __shfl_up_sync(0xffffffffu, orow, 1);
                            const bool starts = orow >= 0 && (lane == 0 || prev != orow - 1);
                            unsigned smask = __ballot_sync(0xffffffffu, starts);
                            const unsigned vm = __ballot_sync(0xffffffffu, orow >= 0);
                            while (smask) {
                                const int a = __ffs(smask) - 1;
                                smask &= smask - 1;
                                // run ends before the next start or the next non-stored row
                                const unsigned gaps = ~vm & ~((2u << a) - 1u);  // lanes > a not stored
                                const int nxt_start = smask ? __ffs(smask) - 1 : 32;
                                const int nxt_gap = gaps ? __ffs(gaps) - 1 : 32;
                                const int e = min(nxt_start, nxt_gap);
                                const int r0 = __shfl_sync(0xffffffffu, orow, a);
                                if (lane == 0 && ok)
                                    bulk_store(p.out0 + (size_t)r0 * NO, buf + a * 256, (uint32_t)(e - a) * 256u);
                            }
                        }
                        if (lane == 0) {
                            if (ok) {
                                bulk_commit();
                                bulk_wait_read0();
                            }
                            mbar_arrive(&stg_empty[rq]);
                        }
                    }
                    __syncwarp();
                }
            }
            if (!head_layer) {
                // Publish "chunk j of layer l stored" once every epilogue
                // warp's stores of this item are complete (the quarter-0
                // warps' bulk stores).
                if (quarter == 0 && lane == 0) bulk_wait0();
                __syncwarp();
                if (lane == 0) mbar_arrive(&item_done[done_n & 3]);
                if (warp == 4 && lane == 0) {
                    if (!mbar_wait(&item_done[done_n & 3], (done_n >> 2) & 1, WAIT_LIM)) {
                        fail(83);
                    } else {
                        fence_proxy_async_global();
                        __threadfence();
                        if (fl)
                            st_release_gpu(flags0 + j, 1);
                        else
                            st_release_gpu(p.flags + j, k + 1);
                    }
                }
                ++done_n;
            }
        }
    }

    __syncthreads();
    if (abort_flag && tid == 0) {
        for (int i = 0; i < C::NWIN; ++i) {
            mbar_wait(&win_full[i], 0, 1u << 16);
            mbar_wait(&win_full[i], 1, 1u << 16);
        }
        for (int i = 0; i < C::S; ++i) {
            mbar_wait(&w_full[i], 0, 1u << 16);
            mbar_wait(&w_full[i], 1, 1u << 16);
        }
    }
    __syncthreads();
    tc_fence_after();
    if (warp == 1) tmem_dealloc(tmem, 512);
    if (warp == 1) tmem_relinquish();
    // The last CTA to leave (every other one has left its loops, so nothing
    // reads the flags any more) zeroes the flags and counters for the next
    // launch: no memset between launches.  CTAs that gave up after a timeout
    // leave through here too.
    const int n5L = p.rows5 > 0 ? (p.rows5 + C::TP5 - 1) / C::TP5 : 0;
    int *const exit_ctr = flags0 + n5L;
    int &last_out = ctl.last_out;
    if (tid == 0) {
        __threadfence();
        last_out = atomicAdd(exit_ctr, 1) == (int)gridDim.x - 1;
        if (last_out) __threadfence();
    }
    __syncthreads();
    if (last_out)
        for (int i = tid; i <= n3L + 1 + n5L; i += blockDim.x) p.flags[i] = 0;
}
#undef WAIT_LIM

// ------------------------------------------------------------------ launch

template <class K, int SMEM>
static int set_attr(K kern) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
    if (e != cudaSuccess) {
        lg_set_error("cudaFuncSetAttribute: %s", cudaGetErrorString(e));
        return LG_ERR_CUDA;
    }
    return LG_OK;
}

// Raises the dynamic shared-memory limit of every instantiation; called once
// per device before any launch (and so before any stream capture).
int tc_init_device() {
    int rc = 0;
#define LG_A(N_, H_, K_, HD_) \
    if (!rc) rc = set_attr<decltype(&tc_conv_kernel<N_, H_, K_, HD_>), TcCfg<N_, H_, K_>::SMEM>(tc_conv_kernel<N_, H_, K_, HD_>);
#define LG_T(H_, K_, HD_) \
    if (!rc) rc = set_attr<decltype(&tc_convT_kernel<H_, K_, HD_>), TcTCfg<H_, K_>::SMEM>(tc_convT_kernel<H_, K_, HD_>);
    LG_A(64, 1, 0, false) LG_A(64, 1, 0, true) LG_A(64, 2, 1, false) LG_A(64, 3, 1, false)
    LG_A(128, 3, 1, false) LG_A(128, 2, 0, false) LG_A(128, 2, 0, true) LG_A(128, 2, 1, false)
    LG_T(2, 0, false) LG_T(2, 0, true) LG_T(2, 1, false)
#define LG_TR(HD_, F_) \
    if (!rc) rc = set_attr<decltype(&tc_trunk_kernel<HD_, F_>), TrunkCfg::SMEM>(tc_trunk_kernel<HD_, F_>);
    LG_TR(false, false) LG_TR(true, false) LG_TR(false, true) LG_TR(true, true)
#undef LG_TR
#undef LG_A
#undef LG_T
    return rc;
}

// Parts the fused head writes: four (one per TMEM lane quarter) for the
// transposed 128-wide kernels and the trunk, one for the 128-row kernel
// (variant 1) and the 64-wide nets (kernel A sums all channels per row).
int tc_head_parts(int n, int variant) { return (n == 128 && variant != 1) ? 4 : 1; }

size_t trunk_flag_ints(int rows, int rows5) {
    // chunk flags, item counter, first-layer chunk flags, exit counter
    return (size_t)(rows + TrunkCfg::TP - 1) / TrunkCfg::TP + 1 + (size_t)(rows5 + TrunkCfg::TP5 - 1) / TrunkCfg::TP5 +
           1;
}

int trunk_layer_item(int rows, int rows5, int k) {
    return (rows5 + TrunkCfg::TP5 - 1) / TrunkCfg::TP5 + k * ((rows + TrunkCfg::TP - 1) / TrunkCfg::TP);
}

template <int N, int HALVES, int KIND, bool HEAD>
static int launch_a(const TcLayer &L, TcParams p, cudaStream_t s, int sm_count) {
    using Cfg = TcCfg<N, HALVES, KIND>;
    CUtensorMap in_map, w_map;
    int rc = encode_map_2d_bf16(&in_map, L.in, (uint64_t)HALVES * 64, (uint64_t)L.rows, 64, Cfg::WROWS);
    if (!rc) rc = encode_map_2d_bf16(&w_map, L.w, 64, (uint64_t)Cfg::NTAPS * HALVES * N, 64, N);
    if (rc) return rc;
    p.ntiles = (L.rows + 127) / 128;
    int grid = std::min(p.ntiles, sm_count);
    tc_conv_kernel<N, HALVES, KIND, HEAD><<<grid, kTcThreads, Cfg::SMEM, s>>>(in_map, w_map, p);
    return LG_OK;
}

template <int HALVES, int KIND, bool HEAD>
static int launch_t(const TcLayer &L, TcParams p, cudaStream_t s, int sm_count) {
    using Cfg = TcTCfg<HALVES, KIND>;
    CUtensorMap in_map, w_map, out_map;
    std::memset(&out_map, 0, sizeof out_map);
    int rc = encode_map_2d_bf16(&in_map, L.in, (uint64_t)HALVES * 64, (uint64_t)L.rows, 64, Cfg::SUBROWS);
    if (!rc) rc = encode_map_2d_bf16(&w_map, L.w, 64, (uint64_t)Cfg::NTAPS * HALVES * 128, 64, 128);
    if (!rc && Cfg::STAGED && !HEAD)
        rc = encode_map_2d_bf16(&out_map, p.out, 128, (uint64_t)L.rows, 128, 32, /*swizzle=*/false);
    if (rc) return rc;
    p.ntiles = (L.rows + 31) / 32;  // 32-row blocks, split evenly over the CTAs
    int grid = std::min(p.ntiles, sm_count);
    tc_convT_kernel<HALVES, KIND, HEAD><<<grid, kTcThreadsT, Cfg::SMEM, s>>>(in_map, w_map, out_map, p);
    return LG_OK;
}

int launch_tc_trunk(const TcTrunk &T, float *parts, size_t part_stride, int *flags, int *err,
                    cudaStream_t s, int sm_count) {
    using C0 = TrunkCfg::C0;
    using C1 = TrunkCfg::C1;
    const bool fused = T.buf5 != nullptr;
    if (T.nl < 1 || T.rows <= 0 || (T.head_w && !parts) || (fused && (T.rows5 <= 0 || !T.w0 || !T.bias0))) {
        lg_set_error("launch_tc_trunk: bad arguments");
        return LG_ERR_ARG;
    }
    CUtensorMap in_a, in_b, out_a, out_b, w_map, in5, w0_map, out_a_sw, out_b_sw;
    int rc = encode_map_2d_bf16(&in_a, T.buf_a, 128, (uint64_t)T.rows, 64, C0::SUBROWS);
    if (!rc) rc = encode_map_2d_bf16(&in_b, T.buf_b, 128, (uint64_t)T.rows, 64, C0::SUBROWS);
    if (!rc) rc = encode_map_2d_bf16(&out_a, T.buf_a, 128, (uint64_t)T.rows, 128, 32, false);
    if (!rc) rc = encode_map_2d_bf16(&out_b, T.buf_b, 128, (uint64_t)T.rows, 128, 32, false);
    // the fragment-path epilogue's stores: 64-channel boxes from 128-byte
    // swizzled staging halves
    if (!rc) rc = encode_map_2d_bf16(&out_a_sw, T.buf_a, 128, (uint64_t)T.rows, 64, 32, true);
    if (!rc) rc = encode_map_2d_bf16(&out_b_sw, T.buf_b, 128, (uint64_t)T.rows, 64, 32, true);
    if (!rc) rc = encode_map_2d_bf16(&w_map, T.w, 64, (uint64_t)T.nl * C0::NTAPS * 2 * 128, 64, 128);
    if (fused) {
        if (!rc) rc = encode_map_2d_bf16(&in5, T.buf5, 128, (uint64_t)T.rows5, 64, TrunkCfg::SUB5);
        if (!rc) rc = encode_map_2d_bf16(&w0_map, T.w0, 64, (uint64_t)C1::NTAPS * 2 * 128, 64, 128);
    } else {
        in5 = in_a;  // unused
        w0_map = w_map;
    }
    if (rc) return rc;
    TrunkParams p{};
    p.bias = T.bias;
    p.scale = T.scale;
    p.bias0 = T.bias0;
    p.scale0 = T.scale0;
    p.head_w = T.head_w;
    p.out0 = (__nv_bfloat16 *)T.buf_a;
    p.act = T.act;
    p.rows = T.rows;
    p.rows5 = fused ? T.rows5 : 0;
    p.nl = T.nl;
    p.parts = parts;
    p.part_stride = part_stride;
    p.count = T.count;
    p.count_base = T.count_base;
    p.flags = flags;
    p.err = err;
    p.wait_limit = T.wait_limit ? T.wait_limit : kWaitLimit;
    p.poll_limit = T.poll_limit ? T.poll_limit : kFlagPolls;
    p.stall_item = T.stall_item;
    const int n3 = (T.rows + TrunkCfg::TP - 1) / TrunkCfg::TP;
    const int n5 = fused ? (T.rows5 + TrunkCfg::TP5 - 1) / TrunkCfg::TP5 : 0;
    const int grid = std::min(n5 + T.nl * n3, sm_count);
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kTrunkThreads);
    cfg.dynamicSmemBytes = TrunkCfg::SMEM;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    if (T.pdl) {
        // No co-residency is needed (items are claimed in order, so every
        // item a claimed item waits for belongs to a running CTA): the
        // launch may start while the previous kernel's CTAs still run.
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
    } else {
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
    }
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e;
    if (T.f16)
        e = T.head_w ? cudaLaunchKernelEx(&cfg, tc_trunk_kernel<true, true>, in_a, in_b, out_a, out_b, w_map, in5,
                                          w0_map, out_a_sw, out_b_sw, p)
                     : cudaLaunchKernelEx(&cfg, tc_trunk_kernel<false, true>, in_a, in_b, out_a, out_b, w_map, in5,
                                          w0_map, out_a_sw, out_b_sw, p);
    else
        e = T.head_w ? cudaLaunchKernelEx(&cfg, tc_trunk_kernel<true, false>, in_a, in_b, out_a, out_b, w_map, in5,
                                          w0_map, out_a_sw, out_b_sw, p)
                     : cudaLaunchKernelEx(&cfg, tc_trunk_kernel<false, false>, in_a, in_b, out_a, out_b, w_map, in5,
                                          w0_map, out_a_sw, out_b_sw, p);
    if (e != cudaSuccess) {
        lg_set_error("trunk launch: %s", cudaGetErrorString(e));
        return LG_ERR_CUDA;
    }
    return LG_OK;
}

size_t tc_conv_smem_bytes(int n, int ntaps, int cin_halves) {
    if (n == 128 && cin_halves == 2) return ntaps == 9 ? TcTCfg<2, 0>::SMEM : TcTCfg<2, 1>::SMEM;
    if (n == 128) return TcCfg<128, 3, 1>::SMEM;
    return ntaps == 9 ? TcCfg<64, 1, 0>::SMEM : TcCfg<64, 2, 1>::SMEM;
}

int launch_tc_conv(const TcLayer &L, __nv_bfloat16 *out_l3, float *parts, size_t part_stride,
                   int *err, cudaStream_t s, int sm_count) {
    TcParams p{};
    p.f16 = L.f16;
    p.bias = L.bias;
    p.scale = L.scale;
    p.head_w = L.head_w;
    p.act = L.act;
    p.rows = L.rows;
    p.out = out_l3;
    p.parts = parts;
    p.part_stride = part_stride;
    p.err = err;
    const bool head = L.head_w != nullptr;
    if ((head && (!parts || L.in_kind != 0)) || (!head && !out_l3) || L.rows <= 0) {
        lg_set_error("launch_tc_conv: bad layer arguments");
        return LG_ERR_ARG;
    }
    if (L.n == 128 && L.cin_halves == 2 && L.in_kind == 0 && L.variant == 1)
        return head ? launch_a<128, 2, 0, true>(L, p, s, sm_count) : launch_a<128, 2, 0, false>(L, p, s, sm_count);
    if (L.n == 128 && L.cin_halves == 2 && L.in_kind == 1 && !head && L.variant == 1)
        return launch_a<128, 2, 1, false>(L, p, s, sm_count);
    if (L.n == 128 && L.cin_halves == 2 && L.in_kind == 0)
        return head ? launch_t<2, 0, true>(L, p, s, sm_count) : launch_t<2, 0, false>(L, p, s, sm_count);
    if (L.n == 128 && L.cin_halves == 2 && L.in_kind == 1 && !head)
        return launch_t<2, 1, false>(L, p, s, sm_count);
    if (L.n == 128 && L.cin_halves == 3 && L.in_kind == 1 && !head)
        return launch_a<128, 3, 1, false>(L, p, s, sm_count);
    if (L.n == 64 && L.cin_halves == 1 && L.in_kind == 0)
        return head ? launch_a<64, 1, 0, true>(L, p, s, sm_count) : launch_a<64, 1, 0, false>(L, p, s, sm_count);
    if (L.n == 64 && L.cin_halves == 2 && L.in_kind == 1 && !head)
        return launch_a<64, 2, 1, false>(L, p, s, sm_count);
    if (L.n == 64 && L.cin_halves == 3 && L.in_kind == 1 && !head)
        return launch_a<64, 3, 1, false>(L, p, s, sm_count);
    lg_set_error("no tensor-core kernel for N=%d halves=%d kind=%d", L.n, L.cin_halves, L.in_kind);
    return LG_ERR_ARG;
}

// ------------------------------------------------------------ tensor maps

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// (FP16 activations and weights move through the same maps: tiled copies do
// not convert, the element type only fixes the 2-byte element size.)
int encode_map_2d_bf16(CUtensorMap *map, const void *base, uint64_t inner, uint64_t rows,
                       uint32_t box_inner, uint32_t box_rows, bool swizzle128) {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void *f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                             &q) != cudaSuccess ||
            !f) {
            lg_set_error("cuTensorMapEncodeTiled not available");
            return LG_ERR_CUDA;
        }
        fn = (EncodeTiledFn)f;
    }
    cuuint64_t dims[2] = {inner, rows};
    cuuint64_t strides[1] = {inner * 2};
    cuuint32_t box[2] = {box_inner, box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides,
                    box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        lg_set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return LG_ERR_CUDA;
    }
    return LG_OK;
}

}  // namespace lg

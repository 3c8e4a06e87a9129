// fast_net.cu -- the distilled student net served in BF16 by one fused
// kernel, and the device-side entropy gate that hands uncertain positions to
// the full nets.
//
// The reference has no learned fast path: its search evaluates every leaf
// with the full policy and value nets (UCTNode.cpp:74-121, 316-344;
// Network.cpp:590-674).  The student (5x5 c_in -> 64, n3x3 x 3x3 64 -> 64,
// ReLU; a 1x1 policy head and a 1x1 value head on the same trunk) is small
// enough that a layer-per-launch schedule is all overhead, so one kernel
// runs the whole trunk with the activations never leaving shared memory:
//
//   * layout: a board is 420 rows of pitch 20 (19 points + a zero column)
//     and 21 rows (19 + two zero rows), so both the 3x3 taps (row shifts
//     20*dy + dx) and the 5x5 first layer's vertical taps (shifts 20*dy,
//     |dy| <= 2) stay inside the board or land on its zero rows.  Rows are
//     128 bytes (64 BF16 channels) in the 128-byte swizzled form the tensor
//     core reads, with 40 rows of margin before and after: 592 rows (74 KB)
//     per board;
//   * two boards ("slots") are in flight per CTA, each with its own buffer
//     and its own 256 TMEM columns: the MMA thread issues layer l of slot 0,
//     layer l of slot 1, layer l + 1 of slot 0, ..., so one slot's epilogue
//     (or plane staging) runs while the tensor core works on the other's;
//   * the MMA: M = 128 rows (4 tiles cover a board), N = 64 output
//     channels, K = 16 per instruction; A = the activation rows read at the
//     tap's row shift, B = one tap's weights (64 x 64, 8 KB) streamed by TMA
//     through a ring of 4 stages.  Taps are the outer loop within a job, so
//     all 4 tile accumulators of the slot are live together;
//   * the first layer is the 5x5 conv as 5 vertical taps over rows that
//     hold the 5 horizontal taps x c_in planes side by side (channel
//     dx * c_in + c = plane c at (y, x + dx - 2)), 128 channels staged in
//     two 64-channel halves: a slot's second half is staged once its first
//     half's MMAs have completed;
//   * each layer's epilogue (TMEM -> + bias -> ReLU -> BF16) writes its
//     output back into the slot's buffer in place: it runs only after every
//     MMA of that slot's layer has completed, and the slot's next layer
//     starts once all epilogue warps have written and fenced their rows;
//   * the last layer's epilogue applies both 1x1 heads to its row and
//     writes two partial sums per head (one per 32-channel half) to global
//     memory; the softmax and the value FC run as the library's finish
//     kernels, which add the parts in a fixed order.
//
// Warps: 0 = TMA producer of the weight slices, 1 = TMEM owner and MMA
// issuer (one thread), 2..9 = plane staging, epilogue (two warps per TMEM
// lane quarter, 32 channels each).  Every wait is bounded; a wait that runs
// out records an error word, and the CTA drains what it issued and frees
// its tensor memory.
#include "lg_kernels.h"

#include <cfloat>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

namespace lg {

using namespace ptx;

namespace {

constexpr int kFW = 64;                              // trunk width
constexpr int kFSlots = 2;                           // boards in flight per CTA
constexpr int kFPitch = 20;
constexpr int kFRowsB = 21 * kFPitch;                // 420 rows per board
constexpr int kFTiles = (kFRowsB + 127) / 128;       // 4 row tiles per board
constexpr int kFPre = 40;                            // margin rows before / after
constexpr int kFBufRows = kFPre + kFTiles * 128 + kFPre;  // 592
constexpr int kFBufBytes = kFBufRows * 128;
constexpr int kFStages = 4;
constexpr int kFSlice = kFW * 128;                   // 64 outputs x 64 K, BF16
constexpr int kFMaxCin = 24;
constexpr int kFMaxLayers = 17;                      // first layer + up to 16 3x3
constexpr int kFEpiWarps = 8;
constexpr int kFEpiThreads = kFEpiWarps * 32;
constexpr int kFThreads = 64 + kFEpiThreads;         // 320
constexpr uint32_t kFWaitLimit = 1u << 26;

constexpr int OFF_BUF = 0;                                             // kFSlots x 592 rows
constexpr int OFF_WST = OFF_BUF + kFSlots * kFBufBytes;                // 151,552
constexpr int OFF_PL = OFF_WST + kFStages * kFSlice;                   // planes of a group
constexpr int OFF_MASK = OFF_PL + ((kFSlots * kFMaxCin * kPoints + 127) / 128) * 128;
constexpr int OFF_LUT = OFF_MASK + ((kFSlots * kPoints * 4 + 127) / 128) * 128;
constexpr int OFF_BIAS = OFF_LUT + 256 * 16;
constexpr int OFF_HEAD = OFF_BIAS + kFMaxLayers * kFW * 4;
constexpr int SMEM_USED = OFF_HEAD + 2 * kFW * 4;
constexpr int kFSmem = 1024 + SMEM_USED;
static_assert(kFBufBytes % 1024 == 0 && OFF_WST % 1024 == 0, "buffers keep the 1024-byte swizzle alignment");
static_assert(kFSmem <= 227 * 1024, "shared memory budget");
static_assert(kFSlots * kFTiles * kFW <= 512, "accumulators fit the tensor memory");

struct FastParams {
    const uint8_t *planes;   // [B][c_in][361]
    int B, c_in, n3;         // positions, input planes, 3x3 layers
    const float *bias;       // [n3 + 1][64]
    const float *wp, *wv;    // [64] policy / value head weights
    float *parts_p, *parts_v;  // [2][part_stride]: head sums over channels 0..31 / 32..63
    size_t part_stride;
    int *err;
    uint32_t wait_limit;
};

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// ReLU, round to nearest even and pack: lo in bits 0..15, hi in 16..31.
__device__ __forceinline__ uint32_t relu_bf16x2(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}

// The MMAs of one weight slice against a board's 4 row tiles: A = the
// buffer rows from descriptor a0 on (tile t 128 rows further: 1024 units of
// 16 bytes), B = the slice at b0; K steps of 16 channels = 32 bytes = 2
// units.  The descriptors are a base plus compile-time offsets, so the
// issuing thread spends an add per operand and MMA.  FIRST: the slice
// starts every accumulator.
template <bool FIRST>
__device__ __forceinline__ void fast_slice(uint32_t tmem, uint64_t a0, uint64_t b0, uint32_t idesc) {
#pragma unroll
    for (int t = 0; t < kFTiles; ++t)
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
            mma_bf16(tmem + (uint32_t)(kFW * t), a0 + (uint64_t)(t * 1024 + 2 * kk), b0 + (uint64_t)(2 * kk), idesc,
                     (FIRST && kk == 0) ? 0u : 1u);
}

// Two boards in flight per CTA, each in its own buffer (slot) and its own
// 256 TMEM columns, so that one board's epilogue (or plane staging) runs
// while the tensor core works on the other's layer: the MMA thread issues
// (layer l, slot 0), (l, slot 1), (l + 1, slot 0), ... and each job waits
// only for its own slot's previous epilogue.
__global__ void __launch_bounds__(kFThreads, 1)
    fast_trunk_kernel(const __grid_constant__ CUtensorMap w_map, const FastParams p) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *buf = smem + OFF_BUF;
    uint8_t *wst = smem + OFF_WST;
    uint8_t *pl = smem + OFF_PL;
    uint32_t *mask = reinterpret_cast<uint32_t *>(smem + OFF_MASK);
    uint4 *lut = reinterpret_cast<uint4 *>(smem + OFF_LUT);
    float *s_bias = reinterpret_cast<float *>(smem + OFF_BIAS);
    float *s_wp = reinterpret_cast<float *>(smem + OFF_HEAD);
    float *s_wv = s_wp + kFW;

    __shared__ uint64_t w_full[kFStages], w_empty[kFStages];
    __shared__ uint64_t stage_full[kFSlots], half_done[kFSlots], acc_full[kFSlots], act_ready[kFSlots];
    __shared__ uint64_t epi_bar, mma_done;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;

    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const int ngroups = (p.B + kFSlots - 1) / kFSlots;
    const int nl = p.n3 + 1;
    const int nslices = 10 + 9 * p.n3;
    const int G = gridDim.x;
    const uint32_t WL = p.wait_limit;

    if (tid == 0) {
        for (int i = 0; i < kFStages; ++i) {
            mbar_init(&w_full[i], 1);
            mbar_init(&w_empty[i], 1);
        }
        for (int i = 0; i < kFSlots; ++i) {
            mbar_init(&stage_full[i], kFEpiWarps);
            mbar_init(&half_done[i], 1);
            mbar_init(&acc_full[i], 1);
            mbar_init(&act_ready[i], kFEpiWarps);
        }
        mbar_init(&epi_bar, kFEpiWarps);
        mbar_init(&mma_done, 1);
        abort_flag = 0;
        fence_mbar_init();
        prefetch_tensormap(&w_map);
    }
    for (int i = tid; i < nl * kFW; i += kFThreads) s_bias[i] = p.bias[i];
    for (int i = tid; i < kFW; i += kFThreads) {
        s_wp[i] = p.wp[i];
        s_wv[i] = p.wv[i];
    }
    // byte -> eight BF16 values 1.0 / 0.0 (bit i -> element i)
    for (int i = tid; i < 256; i += kFThreads) {
        uint32_t w[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            w[k] = (((i >> (2 * k)) & 1) ? 0x3F80u : 0u) | (((i >> (2 * k + 1)) & 1) ? 0x3F800000u : 0u);
        lut[i] = make_uint4(w[0], w[1], w[2], w[3]);
    }
    if (warp == 1) tmem_alloc(&tmem_base, 512);
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;

    auto fail = [&](int code) {
        atomicCAS(p.err, 0, code);
        atomicExch(&abort_flag, 1);
    };
    auto aborted = [&]() { return *(volatile int *)&abort_flag != 0; };

    if (warp == 0) {
        // ------------------------------------------------ weight slices, in
        // the MMA thread's order: first layer (half, slot, tap), then per
        // 3x3 layer (slot, tap)
        if (lane == 0) {
            uint32_t g = 0;
            for (int grp = blockIdx.x; grp < ngroups; grp += G) {
                for (int j = 0; j < kFSlots * nslices; ++j, ++g) {
                    if (aborted()) goto done_producer;
                    int s;
                    if (j < 10 * kFSlots) {
                        const int h = j / (5 * kFSlots), dy = j % 5;
                        s = h * 5 + dy;
                    } else {
                        const int r = j - 10 * kFSlots, l = r / (9 * kFSlots), tap = r % 9;
                        s = 10 + 9 * l + tap;
                    }
                    const int st = g % kFStages;
                    const uint32_t k = g / kFStages;
                    if (!mbar_wait(&w_empty[st], (k & 1) ^ 1, WL)) { fail(91); goto done_producer; }
                    mbar_arrive_expect_tx(&w_full[st], kFSlice);
                    tma_load_2d(wst + st * kFSlice, &w_map, &w_full[st], 0, s * kFW);
                }
            }
        done_producer:;
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(128, kFW);
            const uint64_t b_base = sdesc_sw128(smem_u32(wst));
            uint32_t g = 0, n_stage[kFSlots] = {0, 0}, n_act[kFSlots] = {0, 0};
            for (int grp = blockIdx.x; grp < ngroups; grp += G) {
                // first layer: two 64-channel halves of the expanded rows
                for (int h = 0; h < 2; ++h)
                    for (int sl = 0; sl < kFSlots; ++sl) {
                        if (!mbar_wait(&stage_full[sl], n_stage[sl] & 1, WL)) { fail(92); goto done_mma; }
                        ++n_stage[sl];
                        tc_fence_after();
                        const uint64_t a_base = sdesc_sw128(smem_u32(buf + sl * kFBufBytes));
                        const uint32_t tm = tmem + (uint32_t)(sl * kFTiles * kFW);
                        for (int dy = 0; dy < 5; ++dy, ++g) {
                            const int st = g % kFStages;
                            const uint32_t k = g / kFStages;
                            if (!mbar_wait(&w_full[st], k & 1, WL)) { fail(93); goto done_mma; }
                            tc_fence_after();
                            const uint64_t a0 = a_base + (uint64_t)((kFPre + kFPitch * (dy - 2)) * 8);
                            const uint64_t b0 = b_base + (uint64_t)(st * (kFSlice >> 4));
                            if (h == 0 && dy == 0)
                                fast_slice<true>(tm, a0, b0, idesc);
                            else
                                fast_slice<false>(tm, a0, b0, idesc);
                            mma_commit(&w_empty[st]);
                        }
                        mma_commit(h == 0 ? &half_done[sl] : &acc_full[sl]);
                    }
                for (int l = 1; l < nl; ++l)
                    for (int sl = 0; sl < kFSlots; ++sl) {
                        if (!mbar_wait(&act_ready[sl], n_act[sl] & 1, WL)) { fail(94); goto done_mma; }
                        ++n_act[sl];
                        tc_fence_after();
                        const uint64_t a_base = sdesc_sw128(smem_u32(buf + sl * kFBufBytes));
                        const uint32_t tm = tmem + (uint32_t)(sl * kFTiles * kFW);
                        for (int tap = 0; tap < 9; ++tap, ++g) {
                            const int st = g % kFStages;
                            const uint32_t k = g / kFStages;
                            if (!mbar_wait(&w_full[st], k & 1, WL)) { fail(95); goto done_mma; }
                            tc_fence_after();
                            const int shift = kFPitch * (tap / 3 - 1) + (tap % 3 - 1);
                            const uint64_t a0 = a_base + (uint64_t)((kFPre + shift) * 8);
                            const uint64_t b0 = b_base + (uint64_t)(st * (kFSlice >> 4));
                            if (tap == 0)
                                fast_slice<true>(tm, a0, b0, idesc);
                            else
                                fast_slice<false>(tm, a0, b0, idesc);
                            mma_commit(&w_empty[st]);
                        }
                        mma_commit(&acc_full[sl]);
                    }
            }
        done_mma:
            // every MMA this thread issued has completed before the CTA can
            // free its tensor memory (also after a wait gave up)
            mma_commit(&mma_done);
            mbar_wait(&mma_done, 0, 1u << 20);
        }
    } else {
        // ------------------------------------------------ staging + epilogue
        const int e = tid - 64;
        const int qd = warp & 3;          // TMEM lane quarter this warp may read
        const int chh = (warp - 2) >> 2;  // channels 32*chh .. 32*chh + 31
        const int c_in = p.c_in;
        uint32_t n_half[kFSlots] = {0, 0}, n_acc[kFSlots] = {0, 0}, n_epi = 0;
        auto boards = [&](int grp) { return min(kFSlots, p.B - grp * kFSlots); };

        // barrier of the 8 staging / epilogue warps (bounded)
        auto epi_sync = [&]() -> bool {
            __syncwarp();
            if (lane == 0) mbar_arrive(&epi_bar);
            const bool ok = mbar_wait(&epi_bar, n_epi & 1, WL);
            ++n_epi;
            if (!ok) fail(96);
            return ok;
        };
        auto copy_planes = [&](int grp) {
            const uint8_t *src = p.planes + (size_t)grp * kFSlots * c_in * kPoints;
            const int words = boards(grp) * c_in * kPoints / 4;
            for (int i = e; i < words; i += kFEpiThreads) cp_async4(pl + 4 * i, src + 4 * i);
            cp_async_commit();
        };
        // per point of the group's boards: bit c = plane c (planes already in
        // shared memory); the barriers order it against the staging that
        // reads the masks and the copy that overwrites the planes
        auto build_masks = [&](int grp) -> bool {
            cp_async_wait0();
            if (!epi_sync()) return false;
            const int nb = boards(grp);
            for (int i = e; i < nb * kPoints; i += kFEpiThreads) {
                const int b = i / kPoints, pt = i - b * kPoints;
                const uint8_t *src = pl + (size_t)b * c_in * kPoints + pt;
                uint32_t m = 0;
                for (int c = 0; c < c_in; ++c) m |= (uint32_t)(src[c * kPoints] & 1) << c;
                mask[i] = m;
            }
            return epi_sync();
        };
        // Expanded first-layer rows of slot sl, 64-channel half h, for every
        // buffer row: channel dx * c_in + c = plane c at (y, x + dx - 2);
        // zero rows off the board (and for a slot without a board).
        auto stage = [&](int sl, int h, int nb) {
            uint8_t *sbuf = buf + sl * kFBufBytes;
            const uint32_t *mb = mask + sl * kPoints;
            for (int R = e; R < kFBufRows; R += kFEpiThreads) {
                const int q = R - kFPre;
                uint64_t lo = 0, hi = 0;
                if (sl < nb && q >= 0 && q < kFRowsB) {
                    const int y = q / kFPitch, x = q - y * kFPitch;
                    if (y < kBoard && x < kBoard) {
                        const uint32_t *m = mb + y * kBoard;
#pragma unroll
                        for (int dx = 0; dx < 5; ++dx) {
                            const int xx = x + dx - 2;
                            const uint64_t v = (xx >= 0 && xx < kBoard) ? m[xx] : 0u;
                            const int pos = dx * c_in;
                            if (pos < 64) {
                                lo |= v << pos;
                                if (pos + c_in > 64) hi |= v >> (64 - pos);
                            } else {
                                hi |= v << (pos - 64);
                            }
                        }
                    }
                }
                const uint64_t half = h ? hi : lo;
                uint8_t *row = sbuf + R * 128;
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    *reinterpret_cast<uint4 *>(row + ((j ^ (R & 7)) << 4)) = lut[(half >> (8 * j)) & 0xFF];
            }
        };
        auto stage_done = [&](int sl) {
            fence_proxy_async();
            __syncwarp();
            if (lane == 0) mbar_arrive(&stage_full[sl]);
        };
        // both halves of group grp's first-layer rows, slot by slot, each
        // second half once that slot's first-half MMAs have completed
        auto stage_second_halves = [&](int grp) -> bool {
            for (int sl = 0; sl < kFSlots; ++sl) {
                if (!mbar_wait(&half_done[sl], n_half[sl] & 1, WL)) { fail(97); return false; }
                ++n_half[sl];
                stage(sl, 1, boards(grp));
                stage_done(sl);
            }
            return true;
        };

        const int g0 = blockIdx.x;
        if (g0 < ngroups) {
            copy_planes(g0);
            if (!build_masks(g0)) goto done_epi;
            if (g0 + G < ngroups) copy_planes(g0 + G);
            for (int sl = 0; sl < kFSlots; ++sl) {
                stage(sl, 0, boards(g0));
                stage_done(sl);
            }
            if (!stage_second_halves(g0)) goto done_epi;
            if (g0 + G < ngroups) {
                if (!build_masks(g0 + G)) goto done_epi;
                if (g0 + 2 * G < ngroups) copy_planes(g0 + 2 * G);
            }
        }
        for (int grp = g0; grp < ngroups; grp += G) {
            const int nb = boards(grp);
            const int nxt = grp + G;
            const bool has_next = nxt < ngroups;
            // which of this thread's rows (one per tile) are board points
            uint32_t vmask = 0;
#pragma unroll
            for (int t = 0; t < kFTiles; ++t) {
                const int q = 128 * t + 32 * qd + lane;
                const int y = q / kFPitch, x = q - y * kFPitch;
                if (q < kFRowsB && y < kBoard && x < kBoard) vmask |= 1u << t;
            }
            for (int l = 0; l < nl; ++l) {
                const bool last = l == nl - 1;
                const float *bias = s_bias + l * kFW + chh * 32;
                for (int sl = 0; sl < kFSlots; ++sl) {
                    if (!mbar_wait(&acc_full[sl], n_acc[sl] & 1, WL)) { fail(98); goto done_epi; }
                    ++n_acc[sl];
                    tc_fence_after();
                    const uint32_t vm = sl < nb ? vmask : 0u;
                    const uint32_t t_row = tmem + ((uint32_t)(32 * qd) << 16) +
                                           (uint32_t)(sl * kFTiles * kFW + 32 * chh);
                    uint8_t *sbuf = buf + sl * kFBufBytes;
#pragma unroll
                    for (int t0 = 0; t0 < kFTiles; t0 += 2) {
                        uint32_t v[2][32];
                        tmem_ld32(t_row + (uint32_t)(kFW * t0), v[0]);
                        tmem_ld32(t_row + (uint32_t)(kFW * (t0 + 1)), v[1]);
                        tmem_ld_wait();
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            const int q = 128 * (t0 + u) + 32 * qd + lane;
                            const bool valid = (vm >> (t0 + u)) & 1u;
                            if (!last) {
                                uint32_t w[16];
#pragma unroll
                                for (int i = 0; i < 16; ++i)
                                    w[i] = valid ? relu_bf16x2(__uint_as_float(v[u][2 * i]) + bias[2 * i],
                                                               __uint_as_float(v[u][2 * i + 1]) + bias[2 * i + 1])
                                                 : 0u;
                                const int R = q + kFPre;
                                uint8_t *row = sbuf + R * 128;
#pragma unroll
                                for (int k = 0; k < 4; ++k)
                                    *reinterpret_cast<uint4 *>(row + (((4 * chh + k) ^ (R & 7)) << 4)) =
                                        make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
                            } else {
                                float sp = 0.0f, sv = 0.0f;
#pragma unroll
                                for (int i = 0; i < 32; ++i) {
                                    const float f = fmaxf(__uint_as_float(v[u][i]) + bias[i], 0.0f);
                                    sp = fmaf(f, s_wp[32 * chh + i], sp);
                                    sv = fmaf(f, s_wv[32 * chh + i], sv);
                                }
                                if (valid) {
                                    const int y = q / kFPitch, x = q - y * kFPitch;
                                    const size_t idx = (size_t)(grp * kFSlots + sl) * kPoints + y * kBoard + x;
                                    p.parts_p[chh * p.part_stride + idx] = sp;
                                    p.parts_v[chh * p.part_stride + idx] = sv;
                                }
                            }
                        }
                    }
                    tc_fence_before();
                    if (!last) {
                        fence_proxy_async();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&act_ready[sl]);
                    } else if (has_next) {
                        // this slot's buffer and accumulators are free: the
                        // next group's first half goes in while the tensor
                        // core finishes the other slot
                        stage(sl, 0, boards(nxt));
                        stage_done(sl);
                    }
                }
            }
            if (has_next) {
                if (!stage_second_halves(nxt)) goto done_epi;
                if (nxt + G < ngroups) {
                    if (!build_masks(nxt + G)) goto done_epi;
                    if (nxt + 2 * G < ngroups) copy_planes(nxt + 2 * G);
                }
            }
        }
    done_epi:
        cp_async_wait0();  // no copy into shared memory outlives the CTA
    }

    __syncthreads();
    if (aborted() && tid == 0) {
        // wait (bounded) for weight loads still in flight into this CTA
        for (int i = 0; i < kFStages; ++i) {
            mbar_wait(&w_full[i], 0, 1u << 16);
            mbar_wait(&w_full[i], 1, 1u << 16);
        }
    }
    __syncthreads();
    if (warp == 1) tmem_dealloc(tmem, 512);
}

// ------------------------------------------------------------- the gate

// Per position: fallback = entropy > threshold; the fallback positions'
// indices in ascending order and their count (one CTA, block-wide scans).
__global__ void __launch_bounds__(1024) gate_compact_kernel(const float *__restrict__ entropy, int B,
                                                            float threshold, uint8_t *__restrict__ fallback,
                                                            int *__restrict__ idx, int *__restrict__ count,
                                                            int *__restrict__ count_out) {
    __shared__ int warp_sum[32];
    __shared__ int base;
    const int tid = threadIdx.x, lane = tid % 32, w = tid / 32;
    if (tid == 0) base = 0;
    __syncthreads();
    for (int b0 = 0; b0 < B; b0 += 1024) {
        const int b = b0 + tid;
        const int f = (b < B && entropy[b] > threshold) ? 1 : 0;
        if (b < B && fallback) fallback[b] = (uint8_t)f;
        const unsigned bal = __ballot_sync(0xffffffffu, f);
        const int before = __popc(bal & ((1u << lane) - 1u));
        if (lane == 0) warp_sum[w] = __popc(bal);
        __syncthreads();
        int off = 0;
        for (int k = 0; k < w; ++k) off += warp_sum[k];
        if (f) idx[base + off + before] = b;
        __syncthreads();
        if (tid == 0) {
            int tot = 0;
            for (int k = 0; k < 32; ++k) tot += warp_sum[k];
            base += tot;
        }
        __syncthreads();
    }
    if (tid == 0) {
        *count = base;
        if (count_out) *count_out = base;
    }
}

// dst[i] = src[idx[i]] for i < *count: `bytes` per position (a multiple of 4).
__global__ void __launch_bounds__(256) gate_gather_kernel(const uint8_t *__restrict__ src, int bytes,
                                                          const int *__restrict__ idx, const int *__restrict__ count,
                                                          uint8_t *__restrict__ dst) {
    const int i = blockIdx.x;
    if (i >= *count) return;
    const uint32_t *s = reinterpret_cast<const uint32_t *>(src + (size_t)idx[i] * bytes);
    uint32_t *d = reinterpret_cast<uint32_t *>(dst + (size_t)i * bytes);
    for (int k = threadIdx.x; k < bytes / 4; k += blockDim.x) d[k] = s[k];
}

// probs[idx[i]] = fprobs[i], value[idx[i]] = fvalue[i] for i < *count.
__global__ void __launch_bounds__(384) gate_scatter_kernel(const float *__restrict__ fprobs,
                                                           const float *__restrict__ fvalue,
                                                           const int *__restrict__ idx,
                                                           const int *__restrict__ count, float *__restrict__ probs,
                                                           float *__restrict__ value) {
    const int i = blockIdx.x;
    if (i >= *count) return;
    const int b = idx[i];
    if (threadIdx.x < kPoints) probs[(size_t)b * kPoints + threadIdx.x] = fprobs[(size_t)i * kPoints + threadIdx.x];
    if (threadIdx.x == 0) value[b] = fvalue[i];
}

}  // namespace

int fast_init_device() {
    cudaError_t e = cudaFuncSetAttribute(fast_trunk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kFSmem);
    if (e != cudaSuccess) {
        lg_set_error("fast_trunk_kernel attribute: %s", cudaGetErrorString(e));
        return LG_ERR_CUDA;
    }
    return LG_OK;
}

int launch_gate(const float *entropy, int B, float threshold, uint8_t *fallback, int *idx, int *count,
                int *count_out, cudaStream_t s) {
    gate_compact_kernel<<<1, 1024, 0, s>>>(entropy, B, threshold, fallback, idx, count, count_out);
    return LG_OK;
}

int launch_gate_gather(const uint8_t *src, int bytes, const int *idx, const int *count, int B, uint8_t *dst,
                       cudaStream_t s) {
    if (bytes % 4) return LG_ERR_ARG;
    gate_gather_kernel<<<B, 256, 0, s>>>(src, bytes, idx, count, dst);
    return LG_OK;
}

int launch_gate_scatter(const float *fprobs, const float *fvalue, const int *idx, const int *count, int B,
                        float *probs, float *value, cudaStream_t s) {
    gate_scatter_kernel<<<B, 384, 0, s>>>(fprobs, fvalue, idx, count, probs, value);
    return LG_OK;
}

}  // namespace lg

// ===========================================================================
// C ABI: lg_fast_*
// ===========================================================================

using namespace lg;

struct lg_fast {
    int device = 0, c_in = 0, n3 = 0, H = 0, max_batch = 0, sm_count = 152;
    __nv_bfloat16 *w = nullptr;  // [10 + 9 n3][64][64]: first layer [half][dy], then [layer][tap]
    float *bias = nullptr;       // [n3 + 1][64]
    float *wp = nullptr, *wv = nullptr;  // [64]
    float bp = 0.0f, bv = 0.0f;
    float *w1s = nullptr, *b1 = nullptr, *w2 = nullptr;  // FC1 sliced [H/64][361][64], b1, w2
    float b2 = 0.0f;
    float *parts = nullptr;      // [4][max_batch * 361]: policy halves, value halves
    float *fcpart = nullptr;
    int *fccnt = nullptr;        // value-head group counters, zero between launches
    float *entropy = nullptr;    // [max_batch]
    int *err = nullptr;
    CUtensorMap w_map{};
    // gated evaluation scratch (allocated on the first lg_gated_device)
    uint8_t *g_planes_p = nullptr, *g_planes_v = nullptr;
    size_t g_bytes_p = 0, g_bytes_v = 0;
    float *g_probs = nullptr, *g_value = nullptr;
    int *g_idx = nullptr, *g_count = nullptr;
    uint8_t *g_fallback = nullptr;
    std::vector<void *> allocs;
    std::mutex mu;
};

namespace {

template <class T>
int fast_alloc(lg_fast *f, T **p, size_t count) {
    if (count == 0) count = 1;
    if (cudaMalloc((void **)p, count * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        lg_set_error("lg_fast: cudaMalloc of %zu bytes failed", count * sizeof(T));
        return LG_ERR_ALLOC;
    }
    f->allocs.push_back(*p);
    return LG_OK;
}

size_t fast_param_count(int c_in, int n3, int H) {
    size_t n = (size_t)kFW * c_in * 25 + kFW;
    n += (size_t)n3 * (kFW * kFW * 9 + kFW);
    n += 2 * (kFW + 1);
    n += (size_t)H * kPoints + H + H + 1;
    return n;
}

uint16_t bf16_bits(float v) { return __bfloat16_as_ushort(__float2bfloat16_rn(v)); }

// Flat student weights (per conv W[O][C][k][k] then b[O]; policy head w, b;
// value head w, b; W1[H][361], b1, W2[H], b2) -> the kernel layouts.
int fast_upload(lg_fast *f, const float *host) {
    const int c_in = f->c_in, n3 = f->n3, H = f->H;
    const int nslices = 10 + 9 * n3;
    std::vector<uint16_t> w((size_t)nslices * kFW * kFW, 0);
    std::vector<float> bias((size_t)(n3 + 1) * kFW);
    const float *src = host;
    // first layer: slice (half h, vertical tap dy), K index j <-> channel
    // 64h + j = dx * c_in + c
    for (int h = 0; h < 2; ++h)
        for (int dy = 0; dy < 5; ++dy)
            for (int o = 0; o < kFW; ++o)
                for (int j = 0; j < 64; ++j) {
                    const int ch = 64 * h + j;
                    if (ch >= 5 * c_in) continue;
                    const int dx = ch / c_in, c = ch % c_in;
                    const float v = src[(((size_t)o * c_in + c) * 5 + dy) * 5 + dx];
                    w[(((size_t)(h * 5 + dy)) * kFW + o) * 64 + j] = bf16_bits(v);
                }
    src += (size_t)kFW * c_in * 25;
    for (int o = 0; o < kFW; ++o) bias[o] = src[o];
    src += kFW;
    for (int l = 0; l < n3; ++l) {
        for (int tap = 0; tap < 9; ++tap)
            for (int o = 0; o < kFW; ++o)
                for (int c = 0; c < kFW; ++c)
                    w[((size_t)(10 + 9 * l + tap) * kFW + o) * 64 + c] =
                        bf16_bits(src[(((size_t)o * kFW + c) * 3 + tap / 3) * 3 + tap % 3]);
        src += (size_t)kFW * kFW * 9;
        for (int o = 0; o < kFW; ++o) bias[(size_t)(l + 1) * kFW + o] = src[o];
        src += kFW;
    }
    std::vector<float> wp(src, src + kFW);
    const float bp = src[kFW];
    src += kFW + 1;
    std::vector<float> wv(src, src + kFW);
    const float bv = src[kFW];
    src += kFW + 1;
    const int slices = (H + 63) / 64;
    std::vector<float> w1s((size_t)slices * kPoints * 64, 0.0f);
    for (int u = 0; u < H; ++u)
        for (int k = 0; k < kPoints; ++k) w1s[((size_t)(u / 64) * kPoints + k) * 64 + u % 64] = src[(size_t)u * kPoints + k];
    src += (size_t)H * kPoints;
    std::vector<float> b1(src, src + H);
    src += H;
    std::vector<float> w2(src, src + H);
    src += H;
    const float b2 = src[0];

    LG_CUDA_TRY(cudaMemcpy(f->w, w.data(), w.size() * 2, cudaMemcpyHostToDevice));
    LG_CUDA_TRY(cudaMemcpy(f->bias, bias.data(), bias.size() * 4, cudaMemcpyHostToDevice));
    LG_CUDA_TRY(cudaMemcpy(f->wp, wp.data(), kFW * 4, cudaMemcpyHostToDevice));
    LG_CUDA_TRY(cudaMemcpy(f->wv, wv.data(), kFW * 4, cudaMemcpyHostToDevice));
    LG_CUDA_TRY(cudaMemcpy(f->w1s, w1s.data(), w1s.size() * 4, cudaMemcpyHostToDevice));
    LG_CUDA_TRY(cudaMemcpy(f->b1, b1.data(), H * 4, cudaMemcpyHostToDevice));
    LG_CUDA_TRY(cudaMemcpy(f->w2, w2.data(), H * 4, cudaMemcpyHostToDevice));
    f->bp = bp;
    f->bv = bv;
    f->b2 = b2;
    return LG_OK;
}

int fast_check_err(lg_fast *f) {
    int h = 0;
    LG_CUDA_TRY(cudaMemcpy(&h, f->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
        cudaMemset(f->err, 0, sizeof(int));
        lg_set_error("lg_fast: a kernel gave up a bounded wait (code %d)", h);
        return LG_ERR_DEVICE;
    }
    return LG_OK;
}

}  // namespace

namespace lg {

// One forward of the student over B positions (B <= max_batch): the fused
// trunk, then softmax (with entropy) and the value FC.  Returns the number
// of kernels launched through *nlaunch.
int fast_forward(lg_fast *f, const uint8_t *planes, int B, float T, float *probs, float *logits, float *value,
                 float *entropy, cudaStream_t s, int *nlaunch) {
    FastParams p{};
    p.planes = planes;
    p.B = B;
    p.c_in = f->c_in;
    p.n3 = f->n3;
    p.bias = f->bias;
    p.wp = f->wp;
    p.wv = f->wv;
    p.part_stride = (size_t)f->max_batch * kPoints;
    p.parts_p = f->parts;
    p.parts_v = f->parts + 2 * p.part_stride;
    p.err = f->err;
    p.wait_limit = kFWaitLimit;
    const int groups = (B + kFSlots - 1) / kFSlots;
    const int grid = groups < f->sm_count ? groups : f->sm_count;
    fast_trunk_kernel<<<grid, kFThreads, kFSmem, s>>>(f->w_map, p);
    HeadIn hp{p.parts_p, 2, p.part_stride, f->bp, 0, LG_ACT_RELU, logits};
    launch_softmax(hp, B, T, probs, s, entropy ? entropy : f->entropy);
    HeadIn hv{p.parts_v, 2, p.part_stride, f->bv, 0, LG_ACT_RELU, nullptr};
    launch_value_fc(hv, B, f->w1s, f->b1, f->w2, f->b2, f->H, LG_ACT_RELU, 0, value, f->fcpart, f->fccnt, s);
    *nlaunch = 3;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        lg_set_error("lg_fast: launch failed: %s", cudaGetErrorString(e));
        return LG_ERR_CUDA;
    }
    return LG_OK;
}

// Scratch of the gated evaluation, allocated on first use for the full
// nets' plane sizes: compacted planes of both nets, the full nets' outputs,
// the fallback indices and their count.
int fast_gate_scratch(lg_fast *f, size_t bytes_p, size_t bytes_v, GateScratch *g) {
    if (f->g_bytes_p < bytes_p || f->g_bytes_v < bytes_v || !f->g_idx) {
        const size_t mb = (size_t)f->max_batch;
        int rc = LG_OK;
        if (f->g_bytes_p < bytes_p) {
            rc = fast_alloc(f, &f->g_planes_p, mb * bytes_p);
            if (!rc) f->g_bytes_p = bytes_p;
        }
        if (!rc && f->g_bytes_v < bytes_v) {
            rc = fast_alloc(f, &f->g_planes_v, mb * bytes_v);
            if (!rc) f->g_bytes_v = bytes_v;
        }
        if (!rc && !f->g_idx) {
            if (!rc) rc = fast_alloc(f, &f->g_probs, mb * kPoints);
            if (!rc) rc = fast_alloc(f, &f->g_value, mb);
            if (!rc) rc = fast_alloc(f, &f->g_count, 1);
            if (!rc) rc = fast_alloc(f, &f->g_fallback, mb);
            if (!rc) rc = fast_alloc(f, &f->g_idx, mb);
        }
        if (rc) return rc;
    }
    g->planes_p = f->g_planes_p;
    g->planes_v = f->g_planes_v;
    g->probs = f->g_probs;
    g->value = f->g_value;
    g->idx = f->g_idx;
    g->count = f->g_count;
    g->fallback = f->g_fallback;
    g->entropy = f->entropy;
    g->max_batch = f->max_batch;
    g->device = f->device;
    g->c_in = f->c_in;
    return LG_OK;
}

std::mutex &fast_mutex(lg_fast *f) { return f->mu; }
int fast_status_word(lg_fast *f) { return fast_check_err(f); }

}  // namespace lg

extern "C" LG_API size_t lg_fast_param_count(int c_in, int n3x3, int fc_hidden) {
    return fast_param_count(c_in, n3x3, fc_hidden);
}

extern "C" LG_API void lg_fast_destroy(lg_fast *f) {
    if (!f) return;
    cudaSetDevice(f->device);
    for (void *p : f->allocs) cudaFree(p);
    delete f;
}

extern "C" LG_API int lg_fast_create(int device, int c_in, int n3x3, int fc_hidden, int max_batch,
                                     const float *weights, lg_fast **out) {
    if (!out || !weights || c_in < 1 || c_in > kFMaxCin || c_in % 4 || n3x3 < 1 || n3x3 > kFMaxLayers - 1 ||
        fc_hidden < 1 || fc_hidden > 1024 || max_batch < 1) {
        lg_set_error("lg_fast_create: bad arguments (c_in a multiple of 4 up to %d, 1..%d 3x3 layers)", kFMaxCin,
                     kFMaxLayers - 1);
        return LG_ERR_ARG;
    }
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        lg_set_error("lg_fast_create: no device %d", device);
        return LG_ERR_ARG;
    }
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
    if (major != 10) {
        lg_set_error("lg_fast_create: the fused student kernel needs an sm_10x GPU (got sm_%d%d)", major, minor);
        return LG_ERR_ARG;
    }
    if (int rc0 = finish_init_device()) return rc0;
    lg_fast *f = new lg_fast();
    f->device = device;
    f->c_in = c_in;
    f->n3 = n3x3;
    f->H = fc_hidden;
    f->max_batch = max_batch;
    cudaDeviceGetAttribute(&f->sm_count, cudaDevAttrMultiProcessorCount, device);
    const int nslices = 10 + 9 * n3x3;
    const int slices = (fc_hidden + 63) / 64;
    int rc = fast_init_device();
    if (!rc) rc = fast_alloc(f, &f->w, (size_t)nslices * kFW * kFW);
    if (!rc) rc = fast_alloc(f, &f->bias, (size_t)(n3x3 + 1) * kFW);
    if (!rc) rc = fast_alloc(f, &f->wp, kFW);
    if (!rc) rc = fast_alloc(f, &f->wv, kFW);
    if (!rc) rc = fast_alloc(f, &f->w1s, (size_t)slices * kPoints * 64);
    if (!rc) rc = fast_alloc(f, &f->b1, fc_hidden);
    if (!rc) rc = fast_alloc(f, &f->w2, fc_hidden);
    if (!rc) rc = fast_alloc(f, &f->parts, 4 * (size_t)max_batch * kPoints);
    if (!rc) rc = fast_alloc(f, &f->fcpart, value_fc_part_floats(max_batch, fc_hidden));
    if (!rc) rc = fast_alloc(f, &f->fccnt, value_fc_counter_ints(max_batch, fc_hidden));
    if (!rc && cudaMemset(f->fccnt, 0, sizeof(int) * value_fc_counter_ints(max_batch, fc_hidden)) != cudaSuccess)
        rc = LG_ERR_CUDA;
    if (!rc) rc = fast_alloc(f, &f->entropy, max_batch);
    if (!rc) rc = fast_alloc(f, &f->err, 1);
    if (!rc && cudaMemset(f->err, 0, sizeof(int)) != cudaSuccess) rc = LG_ERR_CUDA;
    if (!rc) rc = encode_map_2d_bf16(&f->w_map, f->w, 64, (uint64_t)nslices * kFW, 64, kFW);
    if (!rc) rc = fast_upload(f, weights);
    if (rc) {
        lg_fast_destroy(f);
        return rc;
    }
    *out = f;
    return LG_OK;
}

extern "C" LG_API int lg_fast_set_weights(lg_fast *f, const float *weights) {
    if (!f || !weights) {
        lg_set_error("lg_fast_set_weights: bad arguments");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(f->mu);
    cudaSetDevice(f->device);
    return fast_upload(f, weights);
}

extern "C" LG_API int lg_fast_device(lg_fast *f, const uint8_t *planes, int B, float temperature, float *probs,
                                     float *logits, float *value, float *entropy, void *stream) {
    if (!f || !planes || ((uintptr_t)planes & 3) || B < 1 || B > f->max_batch || !probs || !value ||
        !(temperature > 0.0f)) {
        lg_set_error("lg_fast_device: bad arguments (planes 4-byte aligned, 1 <= B <= max_batch, probs and "
                     "value required)");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(f->mu);
    cudaSetDevice(f->device);
    int nl = 0;
    return fast_forward(f, planes, B, temperature, probs, logits, value, entropy, (cudaStream_t)stream, &nl);
}

extern "C" LG_API int lg_fast_status(lg_fast *f, void *stream) {
    if (!f) {
        lg_set_error("lg_fast_status: bad arguments");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(f->mu);
    cudaSetDevice(f->device);
    LG_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    return fast_check_err(f);
}

// finish.cu -- the kernels on either side of a forward: the input packing of
// the tensor-core nets' first layer, and the head finish (softmax over the
// 361 points, the value FC chain).
//
//   * pack: 0/1 input planes [B][C][361] -> the first layer's expanded rows
//     (L5 layout, lg_common.cuh);
//   * softmax (Network.cpp:450-469): one CTA per board, max-subtracted,
//     optionally the entropy;
//   * value head (Network.cpp:395-423, 733-737): for H <= 256 one cluster of
//     CTAs per 16 boards, FC1 split over K halves and 64-unit slices and
//     reduced through distributed shared memory, then b1, activation, FC2
//     and the value map; a split-K kernel with counters for wider heads;
//   * softmax + pack: one launch in which some CTAs pack batch k+1's planes
//     while the others finish batch k.
// A chunked device call runs, per chunk, the trunk and then these launches
// as programmatic dependents (griddepcontrol): the work that needs nothing
// from the trunk (packing the next chunk, staging FC weights) starts on the
// SMs its CTAs leave.
#include "lg_kernels.h"

#include <cooperative_groups.h>

#include <cfloat>
#include <utility>

namespace lg {

// ----------------------------------------------------------------- helpers

template <int NT>
__device__ float block_reduce(float v, bool is_max, float *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        float w = __shfl_xor_sync(0xffffffffu, v, o);
        v = is_max ? fmaxf(v, w) : v + w;
    }
    int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = (lane < NT / 32) ? red[lane] : (is_max ? -FLT_MAX : 0.0f);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            float w = __shfl_xor_sync(0xffffffffu, v, o);
            v = is_max ? fmaxf(v, w) : v + w;
        }
        if (lane == 0) red[0] = v;
    }
    __syncthreads();
    float r = red[0];
    __syncthreads();
    return r;
}

// The head output of one point: the sum of `nparts` partial sums (the
// tensor-core path splits the 1x1 head's channel sum over TMEM lane
// quarters), plus the head bias, then the head activation if any.
// The common part counts (4 and 2) are straight-line code, so that a
// thread's loads of several points are all in flight together; the sum is
// always ((p0 + p1) + p2) + p3.
__device__ __forceinline__ float head_value(const HeadIn &h, int b, int p) {
    const float *q = h.parts + (size_t)b * kPoints + p;
    const size_t ps = h.part_stride;
    float s;
    if (h.nparts == 4) {
        const float p0 = q[0], p1 = q[ps], p2 = q[2 * ps], p3 = q[3 * ps];
        s = ((p0 + p1) + p2) + p3;
    } else if (h.nparts == 2) {
        const float p0 = q[0], p1 = q[ps];
        s = p0 + p1;
    } else {
        s = q[0];
        for (int k = 1; k < h.nparts; ++k) s += q[(size_t)k * ps];
    }
    s += h.head_b;
    return h.head_act ? act_fn(s, h.act) : s;
}

// Boards a launch processes: B, or with a device-side count the first
// *count - count_base of them.
__device__ __forceinline__ int head_boards(const HeadIn &h, int B) {
    return h.count ? min(B, max(0, *h.count - h.count_base)) : B;
}

// ----------------------------------------------------------------- softmax

// Network.cpp:450-469 for board b: alpha = max/T; p = exp(x/T - alpha)/sum,
// one point per thread (384 threads).
constexpr int kSoftmaxThreads = 384;
__device__ __forceinline__ void softmax_board(const HeadIn &h, int b, float temperature, float *__restrict__ probs,
                                              float *__restrict__ entropy, float *red) {
    constexpr int NT = kSoftmaxThreads;
    const int p = threadIdx.x;
    float x = (p < kPoints) ? head_value(h, b, p) : -FLT_MAX;
    if (h.logits_out && p < kPoints) h.logits_out[(size_t)b * kPoints + p] = x;
    float mx = block_reduce<NT>(x, true, red);
    float alpha = mx / temperature;
    float e = (p < kPoints) ? expf((x / temperature) - alpha) : 0.0f;
    float den = block_reduce<NT>(e, false, red);
    if (p < kPoints) probs[(size_t)b * kPoints + p] = e / den;
    if (entropy) {
        // -sum p ln p = ln(den) - sum e z / den, z = x/T - alpha = ln e
        const float ez = (p < kPoints) ? e * ((x / temperature) - alpha) : 0.0f;
        const float s = block_reduce<NT>(ez, false, red);
        if (p == 0) entropy[b] = logf(den) - s / den;
    }
}

__global__ void __launch_bounds__(kSoftmaxThreads) softmax_kernel(const HeadIn h, int B, float temperature,
                                                                  float *__restrict__ probs,
                                                                  float *__restrict__ entropy) {
    __shared__ float red[32];
    ptx::grid_dep_launch();
    ptx::grid_dep_wait();
    const int b = blockIdx.x;
    if (b >= head_boards(h, B)) return;
    softmax_board(h, b, temperature, probs, entropy, red);
}

// --------------------------------------------------------------- value head
//
// innerproduct<361,H> (+act) then innerproduct<H,1>, then tanh, (1+tanh)/2
// (Network.cpp:395-423, 733-737) or no map (value_map 2).  Heads of up to
// 256 hidden units run on clusters (value_fc_cluster_kernel below); wider
// heads on this split-K kernel.
// A CTA computes one FC1 tile: 32 boards x 64 hidden units x one of
// kFcSplit fixed K ranges of the 361 inputs.  The 32 boards' head outputs
// for the range are formed in shared memory from the head partial sums, the
// W1 slice for the range is one contiguous block (W1 is stored sliced,
// w1s[H/64][361][64], zero-padded past H), and each thread accumulates a
// 4-board x 2-unit register tile of pre-activation partial sums, stored as
// pre[split][b][unit].  The rest of the head runs in the CTAs that finish
// last, found by counters that those CTAs reset: per (group, slice), the
// split-K sums, b1, the activation and w2 . hidden over the slice's units;
// per group, the sum over slices, b2 and the value map.  Neither the split
// nor any summation order depends on B or on scheduling, so a board's value
// does not depend on its batch.
constexpr int kFcBoards = 32, kFcUnits = 64, kFcSplit = 8, kFcThreads = 256;
constexpr int kFcK = (kPoints + kFcSplit - 1) / kFcSplit;  // 46
constexpr int kFcXPitch = 36;  // floats; rows 16-byte aligned, 4-way store conflicts at most

struct FcArgs {
    const float *w1s, *b1, *w2;
    float b2;
    int H, Hp, act, value_map;
    float *value, *pre;
    int *cnt;  // [ceil(B / kFcBoards)][slices + 1], zero between launches
};

struct FcSmem {
    float Xs[kFcK][kFcXPitch];
    float Ws[kFcK][kFcUnits];
    int last;
};

// CTA `cta` of the head's grid: group = cta / (slices * kFcSplit), then the
// slice, then the K range.
__device__ void value_fc_cta(const HeadIn &h, int B, const FcArgs &f, int cta, FcSmem &sm) {
    const int tid = threadIdx.x;
    const int slices = f.Hp / kFcUnits;
    const int per_group = slices * kFcSplit;
    const int group = cta / per_group, slice = (cta / kFcSplit) % slices, ks = cta % kFcSplit;
    const int b0 = group * kFcBoards;
    const int Bc = head_boards(h, B);
    if (b0 >= Bc) return;  // every CTA of the group returns here: its counter stays 0
    const int k0 = ks * kFcK, nk = min(kPoints, k0 + kFcK) - k0;
    // W1 slice rows k0 .. k0+nk-1: contiguous, float4 loads
    const float4 *wsrc = reinterpret_cast<const float4 *>(f.w1s + ((size_t)slice * kPoints + k0) * kFcUnits);
    constexpr int kWPer = (kFcK * kFcUnits / 4 + kFcThreads - 1) / kFcThreads;  // 3
    float4 wv[kWPer];
#pragma unroll
    for (int j = 0; j < kWPer; ++j) {
        const int i = tid + kFcThreads * j;
        if (i < nk * (kFcUnits / 4)) wv[j] = wsrc[i];
    }
#pragma unroll
    for (int j = 0; j < kWPer; ++j) {
        const int i = tid + kFcThreads * j;
        if (i < nk * (kFcUnits / 4)) reinterpret_cast<float4 *>(&sm.Ws[0][0])[i] = wv[j];
    }
    // head outputs, read along k for each board: every load of the thread is
    // issued before the first store, so the loop waits out one round trip
    constexpr int kPer = (kFcBoards * kFcK + kFcThreads - 1) / kFcThreads;  // 6
    float xv[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        const int i = tid + kFcThreads * j;
        const int bi = i / nk, kk = i - bi * nk, b = b0 + bi;
        xv[j] = (i < kFcBoards * nk && b < Bc) ? head_value(h, b, k0 + kk) : 0.0f;
    }
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        const int i = tid + kFcThreads * j;
        if (i < kFcBoards * nk) {
            const int bi = i / nk, kk = i - bi * nk, b = b0 + bi;
            sm.Xs[kk][bi] = xv[j];
            if (h.logits_out && slice == 0 && b < Bc) h.logits_out[(size_t)b * kPoints + k0 + kk] = xv[j];
        }
    }
    __syncthreads();
    const int up = tid % 32, bq = tid / 32;  // units 2up, 2up+1; boards 4bq .. 4bq+3
    float acc[4][2] = {};
    for (int kk = 0; kk < nk; ++kk) {
        const float4 x = *reinterpret_cast<const float4 *>(&sm.Xs[kk][4 * bq]);
        const float2 w = *reinterpret_cast<const float2 *>(&sm.Ws[kk][2 * up]);
        acc[0][0] = fmaf(x.x, w.x, acc[0][0]);
        acc[0][1] = fmaf(x.x, w.y, acc[0][1]);
        acc[1][0] = fmaf(x.y, w.x, acc[1][0]);
        acc[1][1] = fmaf(x.y, w.y, acc[1][1]);
        acc[2][0] = fmaf(x.z, w.x, acc[2][0]);
        acc[2][1] = fmaf(x.z, w.y, acc[2][1]);
        acc[3][0] = fmaf(x.w, w.x, acc[3][0]);
        acc[3][1] = fmaf(x.w, w.y, acc[3][1]);
    }
    const int u = slice * kFcUnits + 2 * up;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int b = b0 + 4 * bq + j;
        if (b < Bc)
            *reinterpret_cast<float2 *>(f.pre + ((size_t)ks * B + b) * f.Hp + u) =
                make_float2(acc[j][0], acc[j][1]);
    }
    // The last of the kFcSplit CTAs of this (group, slice) adds the split-K
    // partials of its 32 boards x 64 units in a fixed order, applies b1 and
    // the activation, and reduces w2 . hidden over its 64 units: one partial
    // dot product per (board, slice).  The last slice of the group to get
    // there adds those in slice order, adds b2 and applies the value map.
    int *const cnt = f.cnt + group * (slices + 1);
    __threadfence();
    __syncthreads();
    if (tid == 0) {
        const int done = atomicAdd(&cnt[slice], 1);
        sm.last = done == kFcSplit - 1;
        if (sm.last) {
            __threadfence();
            cnt[slice] = 0;
        }
    }
    __syncthreads();
    if (!sm.last) return;
    float *const dots = f.pre + (size_t)kFcSplit * B * f.Hp;  // [group][slice][32]
    {
        const bool u0 = u < f.H, u1 = u + 1 < f.H;
        const float b10 = u0 ? f.b1[u] : 0.0f, b11 = u1 ? f.b1[u + 1] : 0.0f;
        const float w20 = u0 ? f.w2[u] : 0.0f, w21 = u1 ? f.w2[u + 1] : 0.0f;
        float2 pv[4][kFcSplit];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int b = min(b0 + 4 * bq + j, Bc - 1);
#pragma unroll
            for (int k = 0; k < kFcSplit; ++k)
                pv[j][k] = __ldcg(reinterpret_cast<const float2 *>(f.pre + ((size_t)k * B + b) * f.Hp + u));
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float z0 = b10, z1 = b11;
#pragma unroll
            for (int k = 0; k < kFcSplit; ++k) {
                z0 += pv[j][k].x;
                z1 += pv[j][k].y;
            }
            float d = fmaf(w21, act_fn(z1, f.act), w20 * act_fn(z0, f.act));
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
            if (up == 0) dots[((size_t)group * slices + slice) * kFcBoards + 4 * bq + j] = d;
        }
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) {
        const int done = atomicAdd(&cnt[slices], 1);
        sm.last = done == slices - 1;
        if (sm.last) {
            __threadfence();
            cnt[slices] = 0;
        }
    }
    __syncthreads();
    if (!sm.last || tid >= kFcBoards) return;
    const int b = b0 + tid;
    if (b >= Bc) return;
    float dsum = 0.0f;
    for (int sl = 0; sl < slices; ++sl) dsum += __ldcg(dots + ((size_t)group * slices + sl) * kFcBoards + tid);
    const float x = f.b2 + dsum, t = tanhf(x);
    f.value[b] = f.value_map == 2 ? x : (f.value_map ? (1.0f + t) / 2.0f : t);
}

__global__ void __launch_bounds__(kFcThreads) value_fc_kernel(const HeadIn h, int B, const FcArgs f) {
    __shared__ __align__(16) FcSmem sm;
    ptx::grid_dep_launch();
    ptx::grid_dep_wait();
    value_fc_cta(h, B, f, blockIdx.x, sm);
}

// ------------------------------------------------------------------ packing
//
// planes [B][C][361] bytes -> L5 rows [B*399][halves*64] 16-bit, channel
// dx*C + c = plane c at (y, x + dx - 2); zero rows y = 19, 20 and zero
// channels >= 5C.  A CTA (any number of threads) stages one board's planes
// in shared memory, then writes every 16-byte group of its share (part of
// nparts) of the board's rows once.
constexpr int kPackMaxC = 64;
struct PackSmem {
    uint8_t sp[kPackMaxC * kPoints];
    uint32_t mask[kPoints + 3];
    uint4 lut[256];
};

__device__ void pack_l5_board(const uint8_t *__restrict__ planes, int b, int C, int halves, int f16,
                              __nv_bfloat16 *__restrict__ out, int part, int nparts, PackSmem &sm) {
    const int NT = blockDim.x, tid = threadIdx.x;
    const uint8_t *src = planes + (size_t)b * C * kPoints;
    const int nbytes = C * kPoints;
    if (((uintptr_t)src & 7) == 0) {
        // 8-byte words, four loads in flight per thread before the stores
        const int n8 = nbytes / 8;
        const uint2 *s8 = reinterpret_cast<const uint2 *>(src);
        uint2 *d8 = reinterpret_cast<uint2 *>(sm.sp);
        for (int base = 0; base < n8; base += 4 * NT) {
            uint2 r[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int i = base + j * NT + tid;
                if (i < n8) r[j] = s8[i];
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int i = base + j * NT + tid;
                if (i < n8) d8[i] = r[j];
            }
        }
        for (int i = n8 * 8 + tid; i < nbytes; i += NT) sm.sp[i] = src[i];
    } else {
        for (int i = tid; i < nbytes; i += NT) sm.sp[i] = src[i];
    }
    const int groups = halves * 8;
    __nv_bfloat16 *dst = out + (size_t)b * kL5Board * groups * 8;
    const bool aligned = (C % 8) == 0;  // then a group of 8 channels shares one dx
    // this CTA's rows [r_lo, r_hi) of the board, as 16-byte groups [i0, i1)
    const int rpp = (kL5Board + nparts - 1) / nparts;
    const int r_lo = min(kL5Board, part * rpp), r_hi = min(kL5Board, r_lo + rpp);
    const int i0 = r_lo * groups, i1 = r_hi * groups;
    if (aligned && C <= 32) {
        // Per point a bit mask of its C planes, and a table from 8 bits to
        // 8 values 0 / 1 in the operand type: a 16-byte group of a row is
        // then one mask load, one shift and one table load.  Boards whose
        // planes hold other byte values take the byte-by-byte path below.
        const uint32_t one = f16 ? 0x3C00u : 0x3F80u;
        for (int t = tid; t < 256; t += NT) {
            uint32_t w[4];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                w[k] = (((t >> (2 * k)) & 1) ? one : 0u) | (((t >> (2 * k + 1)) & 1) ? (one << 16) : 0u);
            sm.lut[t] = make_uint4(w[0], w[1], w[2], w[3]);
        }
        __syncthreads();
        uint32_t other = 0;
        for (int pt = tid; pt < kPoints; pt += NT) {
            uint32_t m = 0;
            for (int c = 0; c < C; ++c) {
                const uint32_t v = sm.sp[c * kPoints + pt];
                m |= (v & 1u) << c;
                other |= v > 1u;
            }
            sm.mask[pt] = m;
        }
        if (!__syncthreads_or((int)other)) {
            if (NT % groups == 0) {
                // each thread keeps one 16-byte group (its tap dx and first
                // plane c0) and walks the rows: no division by C or groups
                const int g = tid % groups, rstep = NT / groups;
                const int ch0 = g * 8, dx = ch0 / C, c0 = ch0 - dx * C;
                const bool chan = ch0 < 5 * C;
#pragma unroll 4
                for (int r = r_lo + tid / groups; r < r_hi; r += rstep) {
                    const int y = r / kL5Pitch, x = r - y * kL5Pitch;
                    const int sx = x + dx - 2;
                    const bool in = chan && y < kBoard && sx >= 0 && sx < kBoard;
                    const uint32_t bits = in ? (sm.mask[y * kBoard + sx] >> c0) & 0xFFu : 0u;
                    *reinterpret_cast<uint4 *>(dst + ((size_t)r * groups + g) * 8) = sm.lut[bits];
                }
                return;
            }
            for (int i = i0 + tid; i < i1; i += NT) {
                const int r = i / groups, g = i - (i / groups) * groups;
                const int y = r / kL5Pitch, x = r - y * kL5Pitch;
                const int ch0 = g * 8;
                const int dx = ch0 / C, c0 = ch0 - dx * C;
                const int sx = x + dx - 2;
                const bool in = y < kBoard && ch0 < 5 * C && sx >= 0 && sx < kBoard;
                const uint32_t bits = in ? (sm.mask[y * kBoard + sx] >> c0) & 0xFFu : 0u;
                *reinterpret_cast<uint4 *>(dst + (size_t)i * 8) = sm.lut[bits];
            }
        } else {
            for (int i = i0 + tid; i < i1; i += NT) {
                const int r = i / groups, g = i % groups;
                const int y = r / kL5Pitch, x = r % kL5Pitch;
                const int ch0 = g * 8;
                const int dx = ch0 / C, c0 = ch0 - dx * C;
                const int sx = x + dx - 2;
                const bool in = y < kBoard && ch0 < 5 * C && sx >= 0 && sx < kBoard;
                const uint8_t *col = sm.sp + c0 * kPoints + y * kBoard + sx;
                __align__(16) uint16_t v[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) v[j] = round16(in ? (float)col[j * kPoints] : 0.0f, f16);
                *reinterpret_cast<uint4 *>(dst + (size_t)i * 8) = *reinterpret_cast<const uint4 *>(v);
            }
        }
        return;
    }
    __syncthreads();
    for (int i = i0 + tid; i < i1; i += NT) {
        const int r = i / groups, g = i % groups;
        const int y = r / kL5Pitch, x = r % kL5Pitch;
        __align__(16) uint16_t v[8];
        if (aligned) {
            const int ch0 = g * 8;
            const int dx = ch0 / C, c0 = ch0 - dx * C;
            const int sx = x + dx - 2;
            const bool in = y < kBoard && ch0 < 5 * C && sx >= 0 && sx < kBoard;
            const uint8_t *col = sm.sp + c0 * kPoints + y * kBoard + sx;
#pragma unroll
            for (int j = 0; j < 8; ++j) v[j] = round16(in ? (float)col[j * kPoints] : 0.0f, f16);
        } else {
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int ch = g * 8 + j;
                float val = 0.0f;
                if (y < kBoard && ch < 5 * C) {
                    const int dx = ch / C, c = ch % C;
                    const int sx = x + dx - 2;
                    if (sx >= 0 && sx < kBoard) val = (float)sm.sp[c * kPoints + y * kBoard + sx];
                }
                v[j] = round16(val, f16);
            }
        }
        *reinterpret_cast<uint4 *>(dst + (size_t)i * 8) = *reinterpret_cast<const uint4 *>(v);
    }
}

// Four CTAs per board, each writing a quarter of its rows.
// Launched as a programmatic dependent of a trunk (pdl), it packs while the
// trunk's CTAs leave -- `out` must be rows that trunk does not read -- and
// waits for the trunk only before it exits, so that a kernel which waits for
// this one has the trunk's results too.
constexpr int kPackParts = 4;
__global__ void __launch_bounds__(256) pack_planes_l5_kernel(const uint8_t *__restrict__ planes, int B, int C,
                                                             int halves, int f16, __nv_bfloat16 *__restrict__ out,
                                                             const int *__restrict__ count, int count_base) {
    __shared__ __align__(16) PackSmem sm;
    ptx::grid_dep_launch();
    if (count) ptx::grid_dep_wait();  // the count was written by an earlier kernel
    const int b = blockIdx.x / kPackParts;
    if (b < B && !(count && b >= *count - count_base))
        pack_l5_board(planes, b, C, halves, f16, out, blockIdx.x % kPackParts, kPackParts, sm);
    ptx::grid_dep_wait();
}

// Value head for H <= 256 on thread-block clusters: one cluster of 2 x
// slices CTAs per group of 16 boards, CTA rank r = 2 * slice + half, where
// half selects K range [0, 181) or [181, 361) of the 361 inputs and slice 64
// hidden units.  A CTA stages its W1 block (half x slice, 46 KB) in shared
// memory before it waits for the trunk (the weights do not depend on it),
// then forms its boards' head outputs for its K range and accumulates a
// 2-board x 2-unit register tile per thread.  The partial tiles are reduced
// through distributed shared memory: the half-0 CTA of each slice adds its
// partner's tile (z = b1 + half 0 + half 1), applies the activation and
// reduces w2 . hidden over the slice's units with a fixed shuffle tree;
// rank 0 adds the slices' dot products in slice order, adds b2 and applies
// the value map.  No global round trip between the phases, and no
// summation order depends on B or on scheduling.
constexpr int kFccBoards = 16, kFccK0 = 181, kFccMaxSlices = 4;
constexpr size_t kFccSmem = sizeof(float) * ((size_t)kFccK0 * kFcUnits + (size_t)kFccK0 * kFccBoards +
                                             (size_t)kFccBoards * kFcUnits + kFccBoards);

__global__ void __launch_bounds__(kFcThreads) value_fc_cluster_kernel(const HeadIn h, int B, const FcArgs f) {
    namespace cg = cooperative_groups;
    extern __shared__ __align__(16) float fcc_smem[];
    ptx::grid_dep_launch();
    float *const Ws = fcc_smem;                              // [kFccK0][64]
    float *const Xs = Ws + kFccK0 * kFcUnits;                // [kFccK0][16]
    float *const P = Xs + kFccK0 * kFccBoards;               // [16][64]
    float *const dots = P + kFccBoards * kFcUnits;           // [16]
    cg::cluster_group cl = cg::this_cluster();
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const int rank = (int)cl.block_rank(), ncl = (int)cl.num_blocks();
    const int slice = rank / 2, half = rank % 2;
    const int group = (int)blockIdx.x / ncl, b0 = group * kFccBoards;
    const int k0 = half ? kFccK0 : 0, nk = half ? kPoints - kFccK0 : kFccK0;
    // W1 rows k0 .. k0+nk-1 of the slice: one contiguous block, 16-byte copies
    {
        const float4 *src = reinterpret_cast<const float4 *>(f.w1s + ((size_t)slice * kPoints + k0) * kFcUnits);
        const int n4 = nk * (kFcUnits / 4);
        for (int i = tid; i < n4; i += kFcThreads) {
            const uint32_t dst = (uint32_t)__cvta_generic_to_shared(reinterpret_cast<float4 *>(Ws) + i);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src + i) : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    ptx::grid_dep_wait();  // the head outputs
    const int Bc = head_boards(h, B);
    if (b0 >= Bc) {  // the whole cluster leaves here
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        return;
    }
    // head outputs of the group's boards over this CTA's K range: thread
    // kk < nk reads column k0 + kk of all 16 boards, every load in flight
    // before the first store
    static_assert(kFccK0 <= kFcThreads, "one K column per thread");
    if (tid < nk) {
        float xv[kFccBoards];
#pragma unroll
        for (int bi = 0; bi < kFccBoards; ++bi)
            xv[bi] = b0 + bi < Bc ? head_value(h, b0 + bi, k0 + tid) : 0.0f;
#pragma unroll
        for (int bi = 0; bi < kFccBoards; bi += 4)
            *reinterpret_cast<float4 *>(Xs + tid * kFccBoards + bi) = make_float4(xv[bi], xv[bi + 1], xv[bi + 2], xv[bi + 3]);
        if (h.logits_out && slice == 0) {
#pragma unroll
            for (int bi = 0; bi < kFccBoards; ++bi)
                if (b0 + bi < Bc) h.logits_out[(size_t)(b0 + bi) * kPoints + k0 + tid] = xv[bi];
        }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    // boards 2 warp, 2 warp + 1; units 2 lane, 2 lane + 1 of the slice
    float a00 = 0.0f, a01 = 0.0f, a10 = 0.0f, a11 = 0.0f;
#pragma unroll 4
    for (int kk = 0; kk < nk; ++kk) {
        const float2 x = *reinterpret_cast<const float2 *>(Xs + kk * kFccBoards + 2 * warp);
        const float2 w = *reinterpret_cast<const float2 *>(Ws + kk * kFcUnits + 2 * lane);
        a00 = fmaf(x.x, w.x, a00);
        a01 = fmaf(x.x, w.y, a01);
        a10 = fmaf(x.y, w.x, a10);
        a11 = fmaf(x.y, w.y, a11);
    }
    *reinterpret_cast<float2 *>(P + (2 * warp) * kFcUnits + 2 * lane) = make_float2(a00, a01);
    *reinterpret_cast<float2 *>(P + (2 * warp + 1) * kFcUnits + 2 * lane) = make_float2(a10, a11);
    cl.sync();
    if (half == 0) {
        const float *Pr = cl.map_shared_rank(P, rank + 1);
        const int u = slice * kFcUnits + 2 * lane;
        const bool u0 = u < f.H, u1 = u + 1 < f.H;
        const float b10 = u0 ? f.b1[u] : 0.0f, b11 = u1 ? f.b1[u + 1] : 0.0f;
        const float w20 = u0 ? f.w2[u] : 0.0f, w21 = u1 ? f.w2[u + 1] : 0.0f;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int bl = 2 * warp + j;
            const float2 own = *reinterpret_cast<const float2 *>(P + bl * kFcUnits + 2 * lane);
            const float2 oth = *reinterpret_cast<const float2 *>(Pr + bl * kFcUnits + 2 * lane);
            const float z0 = (b10 + own.x) + oth.x, z1 = (b11 + own.y) + oth.y;
            float d = fmaf(w21, act_fn(z1, f.act), w20 * act_fn(z0, f.act));
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
            if (lane == 0) dots[bl] = d;
        }
    }
    cl.sync();
    if (rank == 0 && tid < kFccBoards && b0 + tid < Bc) {
        float dsum = 0.0f;
        for (int sl = 0; sl < ncl / 2; ++sl) dsum += cl.map_shared_rank(dots, 2 * sl)[tid];
        const float xo = f.b2 + dsum, t = tanhf(xo);
        f.value[b0 + tid] = f.value_map == 2 ? xo : (f.value_map ? (1.0f + t) / 2.0f : t);
    }
    cl.sync();  // shared memory stays until rank 0 has read it
}

// ------------------------------------------------------ finish + next pack
//
// CTAs [0, npack) pack the next batch's planes, `pk_parts` CTAs per board;
// CTA npack + b finishes board b (softmax).  The two jobs touch disjoint
// memory.  Launched as a programmatic dependent of the batch's trunk, the
// CTAs are scheduled on the SMs the trunk's CTAs leave, packing CTAs first
// (they need nothing from the trunk); the softmax CTAs wait for the trunk.
union SoftmaxPackSmem {
    float red[32];
    PackSmem pack;
};

__global__ void __launch_bounds__(kSoftmaxThreads, 5)
    softmax_pack_kernel(const HeadIn h, int B, float temperature, float *__restrict__ probs,
                        float *__restrict__ entropy, int npack, const PackJob pk, int pk_parts) {
    __shared__ __align__(16) SoftmaxPackSmem sm;
    ptx::grid_dep_launch();
    if ((int)blockIdx.x < npack) {
        const int q = blockIdx.x, b = q / pk_parts;
        pack_l5_board(pk.planes, b, pk.C, pk.halves, pk.f16, pk.out, q % pk_parts, pk_parts, sm.pack);
        ptx::grid_dep_wait();  // complete only after the trunk, like the softmax CTAs
        return;
    }
    const int b = blockIdx.x - npack;
    ptx::grid_dep_wait();  // the batch's head outputs
    if (b < head_boards(h, B)) softmax_board(h, b, temperature, probs, entropy, sm.red);
}

// ------------------------------------------------------------ host launchers

namespace {
FcArgs fc_args(int B, const float *w1s, const float *b1, const float *w2, float b2, int H, int act,
               int value_map, float *value, float *part, int *cnt) {
    FcArgs f{};
    f.w1s = w1s;
    f.b1 = b1;
    f.w2 = w2;
    f.b2 = b2;
    f.H = H;
    f.Hp = ((H + kFcUnits - 1) / kFcUnits) * kFcUnits;
    f.act = act;
    f.value_map = value_map;
    f.value = value;
    f.pre = part;
    f.cnt = cnt;
    return f;
}
int fc_ctas(int B, int H) {
    return ((B + kFcBoards - 1) / kFcBoards) * ((H + kFcUnits - 1) / kFcUnits) * kFcSplit;
}
}  // namespace

// A launch, optionally as a programmatic dependent of the previous kernel in
// the stream.
template <typename... Exp, typename... Act>
void launch_ex(void (*kern)(Exp...), int grid, int block, cudaStream_t s, bool pdl, Act &&...args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    if (pdl) {
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
    cudaLaunchKernelEx(&cfg, kern, std::forward<Act>(args)...);
}

void launch_value_fc_cluster(const HeadIn &h, int B, const FcArgs &f, int slices, cudaStream_t s, bool pdl);

void launch_softmax(const HeadIn &h, int B, float temperature, float *probs, cudaStream_t s, float *entropy,
                    bool pdl) {
    launch_ex(softmax_kernel, B, kSoftmaxThreads, s, pdl, h, B, temperature, probs, entropy);
}

void launch_value_fc(const HeadIn &h, int B, const float *w1s, const float *b1, const float *w2, float b2, int H,
                     int act, int value_map, float *value, float *part, int *cnt, cudaStream_t s, bool pdl) {
    const FcArgs f = fc_args(B, w1s, b1, w2, b2, H, act, value_map, value, part, cnt);
    const int slices = (H + kFcUnits - 1) / kFcUnits;
    if (slices > kFccMaxSlices) {
        launch_ex(value_fc_kernel, fc_ctas(B, H), kFcThreads, s, pdl, h, B, f);
        return;
    }
    launch_value_fc_cluster(h, B, f, slices, s, pdl);
}

// The cluster value head (H <= 256).
void launch_value_fc_cluster(const HeadIn &h, int B, const FcArgs &f, int slices, cudaStream_t s, bool pdl) {
    const int ncl = 2 * slices, groups = (B + kFccBoards - 1) / kFccBoards;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(groups * ncl);
    cfg.blockDim = dim3(kFcThreads);
    cfg.dynamicSmemBytes = kFccSmem;
    cfg.stream = s;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = ncl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 2 : 1;
    cudaLaunchKernelEx(&cfg, value_fc_cluster_kernel, h, B, f);
}

int finish_init_device() {
    if (cudaFuncSetAttribute(value_fc_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFccSmem) !=
        cudaSuccess) {
        lg_set_error("value head: shared memory attribute: %s", cudaGetErrorString(cudaGetLastError()));
        return LG_ERR_CUDA;
    }
    return LG_OK;
}

size_t value_fc_part_floats(int B, int H) {
    const size_t slices = (H + kFcUnits - 1) / kFcUnits, groups = (B + kFcBoards - 1) / kFcBoards;
    return (size_t)kFcSplit * B * slices * kFcUnits + groups * slices * kFcBoards;
}

size_t value_fc_counter_ints(int B, int H) {
    return (size_t)((B + kFcBoards - 1) / kFcBoards) * ((H + kFcUnits - 1) / kFcUnits + 1);
}

int value_fc_slice_units() { return kFcUnits; }

void launch_pack_planes_l5(const uint8_t *planes, int B, int C, int halves, bool f16, __nv_bfloat16 *out,
                           cudaStream_t s, const int *count, int count_base, bool pdl) {
    launch_ex(pack_planes_l5_kernel, B * kPackParts, 256, s, pdl, planes, B, C, halves, f16 ? 1 : 0, out, count,
              count_base);
}

void launch_finish_pack(const FinishJob &j, const PackJob &pk, cudaStream_t s, bool pdl) {
    if (!j.value_head) {
        // one board per packing CTA: with the softmax CTAs the launch stays
        // one wave at batch 256 (5 resident CTAs per SM)
        const int parts = 1, npack = pk.B * parts;
        launch_ex(softmax_pack_kernel, npack + j.B, kSoftmaxThreads, s, pdl, j.h, j.B, j.temperature, j.probs,
                  j.entropy, npack, pk, parts);
    } else {
        const int slices = (j.H + kFcUnits - 1) / kFcUnits;
        const FcArgs f = fc_args(j.B, j.w1s, j.b1, j.w2, j.b2, j.H, j.act, j.value_map, j.value, j.part, j.cnt);
        // the value head's CTAs run faster in a launch of their own (measured):
        // the packing is a launch before it
        launch_pack_planes_l5(pk.planes, pk.B, pk.C, pk.halves, pk.f16 != 0, pk.out, s, nullptr, 0, pdl);
        if (slices <= kFccMaxSlices)
            launch_value_fc_cluster(j.h, j.B, f, slices, s, pdl);
        else
            launch_ex(value_fc_kernel, fc_ctas(j.B, j.H), kFcThreads, s, pdl, j.h, j.B, f);
    }
}

}  // namespace lg

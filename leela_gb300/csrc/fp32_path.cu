// fp32_path.cu -- the plain FP32 evaluation path (the drop-in path).
//
// Same arithmetic as the reference's BLAS build (Network.cpp:345-423:
// im2col + sgemm + bias + activation, FP32 throughout, expf-based ELU), laid
// out for the GPU:
//   * activations NHWC, [B*361][C] FP32, one board after another;
//   * conv = implicit GEMM  out[m][o] = sum_{tap,c} in[m+tap][c] * W[tap][c][o]
//     with the im2col gather done while staging A tiles in shared memory
//     (no col buffer in HBM), 64x64 output tiles, 4x4 outputs per thread;
//   * small batches split the K loop (taps x channel chunks) across CTAs and
//     reduce the partial sums in a fixed order in a second kernel, so batch 1
//     still fills the GPU and results do not depend on scheduling;
//   * heads: the 1-channel head conv (1x1 or 3x3) is one warp per point; the
//     softmax (Network.cpp:450-469) and the value FC chain
//     (Network.cpp:395-423, 733-737) run one CTA per board.
#include "lg_kernels.h"

#include <cfloat>

namespace lg {

// ----------------------------------------------------------------- helpers

__device__ __forceinline__ float act_fn(float v, int act) {
    // ELU exactly as the reference writes it: x > 0 ? x : exp(x) - 1.
    if (act == LG_ACT_ELU) return (v > 0.0f) ? v : (expf(v) - 1.0f);
    if (act == LG_ACT_RELU) return (v > 0.0f) ? v : 0.0f;
    return v;  // any other code: identity (used by the training kernels)
}

// planes [B][C][361] 0/1 bytes -> NHWC FP32 [B*361][C]
__global__ void pack_planes_f32(const uint8_t *__restrict__ planes, int B, int C,
                                float *__restrict__ out) {
    size_t total = (size_t)B * kPoints * C;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        size_t m = i / C;
        int c = (int)(i % C);
        size_t b = m / kPoints;
        int p = (int)(m % kPoints);
        out[i] = (float)planes[(b * C + c) * kPoints + p];
    }
}

// ------------------------------------------------------- implicit-GEMM conv

constexpr int BM = 64, BN = 64, BKC = 16;

// One K step = one tap and 16 input channels.  Split s covers K steps
// [s*per_split, min((s+1)*per_split, ksteps)).
template <int KS>
__global__ void __launch_bounds__(256) conv_f32_kernel(const float *__restrict__ in,
                                                       const float *__restrict__ wt,
                                                       const float *__restrict__ bias,
                                                       float *__restrict__ out, int M, int C,
                                                       int O, int act, int per_split,
                                                       float *__restrict__ partial) {
    __shared__ float As[BKC][BM + 4];
    __shared__ float Bs[BKC][BN + 4];
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int cchunks = (C + BKC - 1) / BKC;
    const int ksteps = KS * KS * cchunks;
    const int kbeg = blockIdx.z * per_split;
    const int kend = min(ksteps, kbeg + per_split);
    constexpr int PAD = KS / 2;

    // A loader: row ar = tid/4 (0..63), channels ac = (tid%4)*4 .. +3
    const int ar = tid / 4, ac = (tid % 4) * 4;
    const int am = m0 + ar;
    int ab = 0, ay = 0, ax = 0;
    const bool arow_ok = am < M;
    if (arow_ok) {
        ab = am / kPoints;
        int p = am % kPoints;
        ay = p / kBoard;
        ax = p % kBoard;
    }
    // B loader: k row bk = tid/16 (0..15), cols bn = (tid%16)*4
    const int bk = tid / 16, bn = (tid % 16) * 4;

    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;

    for (int ks = kbeg; ks < kend; ++ks) {
        const int tap = ks / cchunks;
        const int c0 = (ks % cchunks) * BKC;
        const int dy = tap / KS - PAD, dx = tap % KS - PAD;
        // stage A
        {
            float v[4] = {0.f, 0.f, 0.f, 0.f};
            int sy = ay + dy, sx = ax + dx;
            if (arow_ok && sy >= 0 && sy < kBoard && sx >= 0 && sx < kBoard) {
                const float *src = in + ((size_t)ab * kPoints + sy * kBoard + sx) * C + c0 + ac;
                if (c0 + ac + 3 < C && (C % 4) == 0) {
                    float4 t = *reinterpret_cast<const float4 *>(src);
                    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
                } else {
#pragma unroll
                    for (int i = 0; i < 4; ++i)
                        if (c0 + ac + i < C) v[i] = src[i];
                }
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) As[ac + i][ar] = v[i];
        }
        // stage B
        {
            float v[4] = {0.f, 0.f, 0.f, 0.f};
            int c = c0 + bk;
            if (c < C) {
                const float *src = wt + ((size_t)tap * C + c) * O + n0 + bn;
                if (n0 + bn + 3 < O && (O % 4) == 0) {
                    float4 t = *reinterpret_cast<const float4 *>(src);
                    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
                } else {
#pragma unroll
                    for (int i = 0; i < 4; ++i)
                        if (n0 + bn + i < O) v[i] = src[i];
                }
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) Bs[bk][bn + i] = v[i];
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BKC; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }

#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int m = m0 + ty + 16 * i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int n = n0 + tx + 16 * j;
            if (n >= O) continue;
            if (partial) {
                partial[((size_t)blockIdx.z * M + m) * O + n] = acc[i][j];
            } else {
                out[(size_t)m * O + n] = act_fn(bias[n] + acc[i][j], act);
            }
        }
    }
}

// Fixed-order reduction of the split-K partial sums, then bias + activation.
__global__ void splitk_reduce_f32(const float *__restrict__ partial, int nsplit, size_t MO, int O,
                                  const float *__restrict__ bias, int act,
                                  float *__restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < MO;
         i += (size_t)gridDim.x * blockDim.x) {
        float s = 0.0f;
        for (int k = 0; k < nsplit; ++k) s += partial[(size_t)k * MO + i];
        out[i] = act_fn(bias[i % O] + s, act);
    }
}

// ---------------------------------------------------------------- head conv

// logits[b][p] = act?(bias + sum_{tap,c} in[b][p+tap][c] * wh[tap][c]); one
// warp per point, lanes over channels.
__global__ void head_conv_f32(const float *__restrict__ in, const float *__restrict__ wh,
                              float bias, int B, int C, int k, int do_act, int act,
                              float *__restrict__ logits) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
    int lane = threadIdx.x % 32;
    if (warp >= B * kPoints) return;
    int b = warp / kPoints, p = warp % kPoints;
    int y = p / kBoard, x = p % kBoard, pad = k / 2;
    float s = 0.0f;
    for (int t = 0; t < k * k; ++t) {
        int sy = y + t / k - pad, sx = x + t % k - pad;
        if (sy < 0 || sy >= kBoard || sx < 0 || sx >= kBoard) continue;
        const float *src = in + ((size_t)b * kPoints + sy * kBoard + sx) * C;
        for (int c = lane; c < C; c += 32) s = fmaf(src[c], wh[t * C + c], s);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        float v = bias + s;
        logits[warp] = do_act ? act_fn(v, act) : v;
    }
}

// ------------------------------------------------------------------- finish

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
__device__ __forceinline__ float head_value(const HeadIn &h, int b, int p) {
    size_t i = (size_t)b * kPoints + p;
    float s = h.parts[i];
    for (int k = 1; k < h.nparts; ++k) s += h.parts[(size_t)k * h.part_stride + i];
    s += h.head_b;
    return h.head_act ? act_fn(s, h.act) : s;
}

// Network.cpp:450-469 per board: alpha = max/T; p = exp(x/T - alpha)/sum.
// Boards a launch processes: B, or with a device-side count the first
// *count - count_base of them.
__device__ __forceinline__ int head_boards(const HeadIn &h, int B) {
    return h.count ? min(B, max(0, *h.count - h.count_base)) : B;
}

__global__ void __launch_bounds__(384) softmax_kernel(const HeadIn h, int B, float temperature,
                                                      float *__restrict__ probs, float *__restrict__ entropy) {
    __shared__ float red[32];
    int b = blockIdx.x;
    if (b >= head_boards(h, B)) return;
    int p = threadIdx.x;
    float x = (p < kPoints) ? head_value(h, b, p) : -FLT_MAX;
    if (h.logits_out && p < kPoints) h.logits_out[(size_t)b * kPoints + p] = x;
    float mx = block_reduce<384>(x, true, red);
    float alpha = mx / temperature;
    float e = (p < kPoints) ? expf((x / temperature) - alpha) : 0.0f;
    float den = block_reduce<384>(e, false, red);
    if (p < kPoints) probs[(size_t)b * kPoints + p] = e / den;
    if (entropy) {
        // -sum p ln p = ln(den) - sum e z / den, z = x/T - alpha = ln e
        const float ez = (p < kPoints) ? e * ((x / temperature) - alpha) : 0.0f;
        const float s = block_reduce<384>(ez, false, red);
        if (p == 0) entropy[b] = logf(den) - s / den;
    }
}

// innerproduct<361,H> (+act) then innerproduct<H,1>, then tanh, (1+tanh)/2
// (Network.cpp:395-423, 733-737) or no map (value_map 2), as a tiled GEMM
// over boards.
// value_fc1_kernel: one CTA = 32 boards x 64 hidden units x one of
// kFcSplit fixed K ranges of the 361 inputs.  The 32 boards' head outputs
// for the range are formed in shared memory from the head partial sums, the
// W1 slice for the range is one contiguous block (W1 is stored sliced,
// w1s[H/64][361][64], zero-padded past H), and each thread accumulates a
// 4-board x 2-unit register tile.  It writes pre-activation partial sums
// pre[split][b][unit].  value_final_kernel adds the kFcSplit partials in a
// fixed order plus b1, applies the activation, reduces w2 . hidden over the
// block in a fixed order, adds b2 and applies the value map.  The split does
// not depend on B, so a board's value does not depend on its batch.
constexpr int kFcBoards = 32, kFcUnits = 64, kFcSplit = 8;
constexpr int kFcK = (kPoints + kFcSplit - 1) / kFcSplit;  // 46
constexpr int kFcXPitch = 36;  // floats; rows 16-byte aligned, 4-way store conflicts at most

__global__ void __launch_bounds__(256) value_fc1_kernel(const HeadIn h, int B,
                                                        const float *__restrict__ w1s, int Hp,
                                                        float *__restrict__ pre) {
    __shared__ __align__(16) float Xs[kFcK][kFcXPitch];
    __shared__ __align__(16) float Ws[kFcK][kFcUnits];
    const int tid = threadIdx.x;
    const int b0 = blockIdx.x * kFcBoards, slice = blockIdx.y, ks = blockIdx.z;
    const int Bc = head_boards(h, B);
    if (b0 >= Bc) return;
    const int k0 = ks * kFcK, nk = min(kPoints, k0 + kFcK) - k0;
    // W1 slice rows k0 .. k0+nk-1: contiguous, float4 loads
    const float4 *wsrc = reinterpret_cast<const float4 *>(w1s + ((size_t)slice * kPoints + k0) * kFcUnits);
    constexpr int kWPer = (kFcK * kFcUnits / 4 + 255) / 256;  // 3
    float4 wv[kWPer];
#pragma unroll
    for (int j = 0; j < kWPer; ++j) {
        const int i = tid + 256 * j;
        if (i < nk * (kFcUnits / 4)) wv[j] = wsrc[i];
    }
#pragma unroll
    for (int j = 0; j < kWPer; ++j) {
        const int i = tid + 256 * j;
        if (i < nk * (kFcUnits / 4)) reinterpret_cast<float4 *>(&Ws[0][0])[i] = wv[j];
    }
    // head outputs, read along k for each board: every load of the thread is
    // issued before the first store, so the loop waits out one round trip
    constexpr int kPer = (kFcBoards * kFcK + 255) / 256;  // 6
    float xv[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        const int i = tid + 256 * j;
        const int bi = i / nk, kk = i - bi * nk, b = b0 + bi;
        xv[j] = (i < kFcBoards * nk && b < Bc) ? head_value(h, b, k0 + kk) : 0.0f;
    }
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        const int i = tid + 256 * j;
        if (i < kFcBoards * nk) {
            const int bi = i / nk, kk = i - bi * nk, b = b0 + bi;
            Xs[kk][bi] = xv[j];
            if (h.logits_out && slice == 0 && b < Bc) h.logits_out[(size_t)b * kPoints + k0 + kk] = xv[j];
        }
    }
    __syncthreads();
    const int up = tid % 32, bq = tid / 32;  // units 2up, 2up+1; boards 4bq .. 4bq+3
    float acc[4][2] = {};
    for (int kk = 0; kk < nk; ++kk) {
        const float4 x = *reinterpret_cast<const float4 *>(&Xs[kk][4 * bq]);
        const float2 w = *reinterpret_cast<const float2 *>(&Ws[kk][2 * up]);
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
            *reinterpret_cast<float2 *>(pre + ((size_t)ks * B + b) * Hp + u) = make_float2(acc[j][0], acc[j][1]);
    }
}

__global__ void __launch_bounds__(256) value_final_kernel(const float *__restrict__ pre, int B, int H, int Hp,
                                                          const float *__restrict__ b1,
                                                          const float *__restrict__ w2, float b2, int act,
                                                          int value_map, float *__restrict__ value,
                                                          const int *__restrict__ count, int count_base) {
    __shared__ float red[32];
    const int b = blockIdx.x;
    if (b >= B || (count && b >= *count - count_base)) return;
    float s = 0.0f;
    for (int u = threadIdx.x; u < H; u += 256) {
        float z = b1[u];
#pragma unroll
        for (int k = 0; k < kFcSplit; ++k) z += pre[((size_t)k * B + b) * Hp + u];
        s = fmaf(w2[u], act_fn(z, act), s);
    }
    s = block_reduce<256>(s, false, red);
    if (threadIdx.x == 0) {
        const float x = b2 + s, t = tanhf(x);
        value[b] = value_map == 2 ? x : (value_map ? (1.0f + t) / 2.0f : t);
    }
}

// ------------------------------------------------------------ host launchers

int conv_f32_splits(int M, int O, int C, int k) {
    int ctas = ((M + BM - 1) / BM) * ((O + BN - 1) / BN);
    int ksteps = k * k * ((C + BKC - 1) / BKC);
    int want = (2 * 152 + ctas - 1) / ctas;
    if (want > ksteps / 2) want = ksteps / 2;
    if (want < 1) want = 1;
    return want;
}

void launch_pack_planes_f32(const uint8_t *planes, int B, int C, float *out, cudaStream_t s) {
    size_t total = (size_t)B * kPoints * C;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    pack_planes_f32<<<blocks, 256, 0, s>>>(planes, B, C, out);
}

void launch_conv_f32(const float *in, const float *wt, const float *bias, float *out, int B,
                     int C, int O, int k, int act, float *partial, cudaStream_t s) {
    int M = B * kPoints;
    int nsplit = conv_f32_splits(M, O, C, k);
    int ksteps = k * k * ((C + BKC - 1) / BKC);
    int per = (ksteps + nsplit - 1) / nsplit;
    nsplit = (ksteps + per - 1) / per;
    dim3 grid((M + BM - 1) / BM, (O + BN - 1) / BN, nsplit);
    float *part = nsplit > 1 ? partial : nullptr;
    switch (k) {
    case 1: conv_f32_kernel<1><<<grid, 256, 0, s>>>(in, wt, bias, out, M, C, O, act, per, part); break;
    case 3: conv_f32_kernel<3><<<grid, 256, 0, s>>>(in, wt, bias, out, M, C, O, act, per, part); break;
    default: conv_f32_kernel<5><<<grid, 256, 0, s>>>(in, wt, bias, out, M, C, O, act, per, part); break;
    }
    if (nsplit > 1) {
        size_t MO = (size_t)M * O;
        int blocks = (int)((MO + 255) / 256);
        if (blocks > 2048) blocks = 2048;
        splitk_reduce_f32<<<blocks, 256, 0, s>>>(partial, nsplit, MO, O, bias, act, out);
    }
}

size_t conv_f32_partial_floats(int B, int C, int O, int k) {
    int M = B * kPoints;
    int nsplit = conv_f32_splits(M, O, C, k);
    int ksteps = k * k * ((C + BKC - 1) / BKC);
    int per = (ksteps + nsplit - 1) / nsplit;
    nsplit = (ksteps + per - 1) / per;
    return nsplit > 1 ? (size_t)nsplit * M * O : 0;
}

void launch_head_conv_f32(const float *in, const float *wh, float bias, int B, int C, int k,
                          int do_act, int act, float *logits, cudaStream_t s) {
    int warps = B * kPoints;
    int blocks = (warps * 32 + 255) / 256;
    head_conv_f32<<<blocks, 256, 0, s>>>(in, wh, bias, B, C, k, do_act, act, logits);
}

void launch_softmax(const HeadIn &h, int B, float temperature, float *probs, cudaStream_t s, float *entropy) {
    softmax_kernel<<<B, 384, 0, s>>>(h, B, temperature, probs, entropy);
}

void launch_value_fc(const HeadIn &h, int B, const float *w1s, const float *b1, const float *w2,
                     float b2, int H, int act, int value_map, float *value, float *part,
                     cudaStream_t s) {
    const int slices = (H + kFcUnits - 1) / kFcUnits;
    dim3 grid((B + kFcBoards - 1) / kFcBoards, slices, kFcSplit);
    value_fc1_kernel<<<grid, 256, 0, s>>>(h, B, w1s, slices * kFcUnits, part);
    value_final_kernel<<<B, 256, 0, s>>>(part, B, H, slices * kFcUnits, b1, w2, b2, act, value_map, value,
                                         h.count, h.count_base);
}

size_t value_fc_part_floats(int B, int H) {
    return (size_t)kFcSplit * B * (((H + kFcUnits - 1) / kFcUnits) * kFcUnits);
}

int value_fc_slice_units() { return kFcUnits; }

}  // namespace lg

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
//   * head: the 1-channel head conv (1x1 or 3x3) is one warp per point; the
//     softmax and the value FC chain that follow are finish.cu's.
#include "lg_kernels.h"

#include <cfloat>

namespace lg {

// ----------------------------------------------------------------- helpers


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

}  // namespace lg

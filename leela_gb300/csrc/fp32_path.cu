// fp32_path.cu -- the plain FP32 evaluation path (the drop-in path).
//
// Same arithmetic as the reference's BLAS build (Network.cpp:345-423:
// im2col + sgemm + bias + activation, FP32 throughout, expf-based ELU), laid
// out for the GPU:
//   * activations NHWC, [B*361][C] FP32, one board after another;
//   * conv = implicit GEMM  out[m][o] = sum_{tap,c} in[m+tap][c] * W[tap][c][o]
//     with the im2col gather done while staging A tiles in shared memory
//     (no col buffer in HBM): 128x128 output tiles with 8x8 outputs per
//     thread and double-buffered K steps for layers of 128k channels,
//     64x64 tiles with 4x4 outputs per thread otherwise;
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

// Layers of 128k output channels: 128 x 128 tiles, 8 x 8 outputs per thread
// (two float4 loads of each operand per 64 FMAs), K steps of one tap and 8
// input channels double-buffered in shared memory, the next step's global
// loads in flight while the current one is multiplied.  Each output is still
// one FMA chain over (tap, channel) in order, as in the 64 x 64 kernel.
constexpr int BM2 = 128, BN2 = 128, BKC2 = 8;

template <int KS>
__global__ void __launch_bounds__(256, 2) conv_f32_big_kernel(const float *__restrict__ in,
                                                              const float *__restrict__ wt,
                                                              const float *__restrict__ bias,
                                                              float *__restrict__ out, int M, int C, int O,
                                                              int act, int per_split, float *__restrict__ partial) {
    __shared__ __align__(16) float As[2][BKC2][BM2 + 4];
    __shared__ __align__(16) float Bs[2][BKC2][BN2 + 4];
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    const int m0 = blockIdx.x * BM2, n0 = blockIdx.y * BN2;
    const int cchunks = (C + BKC2 - 1) / BKC2;
    const int ksteps = KS * KS * cchunks;
    const int kbeg = blockIdx.z * per_split;
    const int kend = min(ksteps, kbeg + per_split);
    constexpr int PAD = KS / 2;
    // A loader: row ar (0..127), channels ac .. ac+3 (ac = 0 or 4)
    const int ar = tid / 2, ac = (tid % 2) * 4;
    const int am = m0 + ar;
    const bool arow_ok = am < M;
    int ab = 0, ay = 0, ax = 0;
    if (arow_ok) {
        ab = am / kPoints;
        const int p = am - ab * kPoints;
        ay = p / kBoard;
        ax = p - ay * kBoard;
    }
    // B loader: k row bk (0..7), columns bn .. bn+3
    const int bk = tid / 32, bn = (tid % 32) * 4;
    const bool vecC = (C % 4) == 0, vecO = (O % 4) == 0;
    auto load_a = [&](int ks) {
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        const int tap = ks / cchunks, c0 = (ks - tap * cchunks) * BKC2;
        const int sy = ay + tap / KS - PAD, sx = ax + tap % KS - PAD;
        if (arow_ok && sy >= 0 && sy < kBoard && sx >= 0 && sx < kBoard) {
            const float *src = in + ((size_t)ab * kPoints + sy * kBoard + sx) * C + c0 + ac;
            if (vecC && c0 + ac + 3 < C) {
                v = *reinterpret_cast<const float4 *>(src);
            } else {
                if (c0 + ac + 0 < C) v.x = src[0];
                if (c0 + ac + 1 < C) v.y = src[1];
                if (c0 + ac + 2 < C) v.z = src[2];
                if (c0 + ac + 3 < C) v.w = src[3];
            }
        }
        return v;
    };
    auto load_b = [&](int ks) {
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        const int tap = ks / cchunks, c = (ks - tap * cchunks) * BKC2 + bk;
        if (c < C) {
            const float *src = wt + ((size_t)tap * C + c) * O + n0 + bn;
            if (vecO && n0 + bn + 3 < O) {
                v = *reinterpret_cast<const float4 *>(src);
            } else {
                if (n0 + bn + 0 < O) v.x = src[0];
                if (n0 + bn + 1 < O) v.y = src[1];
                if (n0 + bn + 2 < O) v.z = src[2];
                if (n0 + bn + 3 < O) v.w = src[3];
            }
        }
        return v;
    };
    auto store = [&](int buf, const float4 &va, const float4 &vb) {
        As[buf][ac + 0][ar] = va.x;
        As[buf][ac + 1][ar] = va.y;
        As[buf][ac + 2][ar] = va.z;
        As[buf][ac + 3][ar] = va.w;
        *reinterpret_cast<float4 *>(&Bs[buf][bk][bn]) = vb;
    };
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
    if (kbeg < kend) {
        store(0, load_a(kbeg), load_b(kbeg));
        __syncthreads();
    }
    for (int ks = kbeg; ks < kend; ++ks) {
        const int cur = (ks - kbeg) & 1;
        const bool more = ks + 1 < kend;
        float4 na, nb;
        if (more) {
            na = load_a(ks + 1);
            nb = load_b(ks + 1);
        }
#pragma unroll
        for (int kk = 0; kk < BKC2; ++kk) {
            const float4 a0 = *reinterpret_cast<const float4 *>(&As[cur][kk][ty * 4]);
            const float4 a1 = *reinterpret_cast<const float4 *>(&As[cur][kk][64 + ty * 4]);
            const float4 b0 = *reinterpret_cast<const float4 *>(&Bs[cur][kk][tx * 4]);
            const float4 b1 = *reinterpret_cast<const float4 *>(&Bs[cur][kk][64 + tx * 4]);
            const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        if (more) store(cur ^ 1, na, nb);
        __syncthreads();
    }
    // rows ty*4 + i and 64 + ty*4 + i, columns tx*4 + j and 64 + tx*4 + j
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int m = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + i - 4);
        if (m >= M) continue;
#pragma unroll
        for (int jh = 0; jh < 2; ++jh) {
            const int n = n0 + jh * 64 + tx * 4;
            float v[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) v[j] = acc[i][jh * 4 + j];
            if (partial) {
                float *dst = partial + ((size_t)blockIdx.z * M + m) * O + n;
                if (vecO && n + 3 < O) {
                    *reinterpret_cast<float4 *>(dst) = make_float4(v[0], v[1], v[2], v[3]);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (n + j < O) dst[j] = v[j];
                }
            } else {
                float *dst = out + (size_t)m * O + n;
                float w[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) w[j] = n + j < O ? act_fn(bias[n + j] + v[j], act) : 0.0f;
                if (vecO && n + 3 < O) {
                    *reinterpret_cast<float4 *>(dst) = make_float4(w[0], w[1], w[2], w[3]);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (n + j < O) dst[j] = w[j];
                }
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

namespace {
// The kernel a layer runs on: 128 x 128 tiles for 128k output channels
// when the rows alone give every SM a tile (no split-K needed), else 64 x 64
// (more, smaller tiles for small batches); tile sizes and channels per K
// step.
struct F32Plan {
    bool big;
    int bm, bn, bkc;
};
F32Plan f32_plan(int M, int O) {
    return (O % BN2 == 0 && M >= 152 * BM2) ? F32Plan{true, BM2, BN2, BKC2} : F32Plan{false, BM, BN, BKC};
}
}  // namespace

int conv_f32_splits(int M, int O, int C, int k) {
    const F32Plan pl = f32_plan(M, O);
    int ctas = ((M + pl.bm - 1) / pl.bm) * ((O + pl.bn - 1) / pl.bn);
    int ksteps = k * k * ((C + pl.bkc - 1) / pl.bkc);
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
    const F32Plan pl = f32_plan(M, O);
    int nsplit = conv_f32_splits(M, O, C, k);
    int ksteps = k * k * ((C + pl.bkc - 1) / pl.bkc);
    int per = (ksteps + nsplit - 1) / nsplit;
    nsplit = (ksteps + per - 1) / per;
    dim3 grid((M + pl.bm - 1) / pl.bm, (O + pl.bn - 1) / pl.bn, nsplit);
    float *part = nsplit > 1 ? partial : nullptr;
    if (pl.big) {
        switch (k) {
        case 1: conv_f32_big_kernel<1><<<grid, 256, 0, s>>>(in, wt, bias, out, M, C, O, act, per, part); break;
        case 3: conv_f32_big_kernel<3><<<grid, 256, 0, s>>>(in, wt, bias, out, M, C, O, act, per, part); break;
        default: conv_f32_big_kernel<5><<<grid, 256, 0, s>>>(in, wt, bias, out, M, C, O, act, per, part); break;
        }
    } else {
        switch (k) {
        case 1: conv_f32_kernel<1><<<grid, 256, 0, s>>>(in, wt, bias, out, M, C, O, act, per, part); break;
        case 3: conv_f32_kernel<3><<<grid, 256, 0, s>>>(in, wt, bias, out, M, C, O, act, per, part); break;
        default: conv_f32_kernel<5><<<grid, 256, 0, s>>>(in, wt, bias, out, M, C, O, act, per, part); break;
        }
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
    const F32Plan pl = f32_plan(M, O);
    int nsplit = conv_f32_splits(M, O, C, k);
    int ksteps = k * k * ((C + pl.bkc - 1) / pl.bkc);
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

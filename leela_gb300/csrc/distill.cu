// distill.cu -- the distilled "student" net: a small policy + value net
// (5x5 c_in->W, n3x3 x 3x3 W->W, ReLU; a 1x1 policy head -> softmax over 361;
// a 1x1 value head -> FC 361->H ReLU -> FC H->1 -> tanh) trained on the GPU
// by the kernels in this file, in FP32.
//
// The reference has no counterpart: it trained its nets offline with Caffe
// (Network.cpp:1381-1509) and evaluates a fixed net per leaf.  The student
// answers leaves first; the caller falls back to the full net when the
// student's policy entropy is high (see leela_gb300/distill.py).
//
// Loss per position: KL(teacher policy || student softmax) + value_weight *
// (tanh output - target value)^2, averaged over the batch.
//
// Layouts (NHWC, [B*361][C] FP32, as the FP32 inference path):
//   conv forward / input gradient  = conv_f32_kernel (fp32_path.cu); the
//     input gradient is the conv of the output gradient with the weights
//     flipped in space and transposed in channels;
//   weight gradient dW[tap][c][o] = sum_m X[m + shift(tap)][c] * dY[m][o]
//     (st_conv_wgrad, 64x64 tiles, split over rows, atomics into dW).
// Parameters live on the device in "GPU layout" (conv W as [tap][cin][cout]);
// lg_student_get/set_params convert to the flat OIHW layout of
// include/leela_gpu.h (so the policy and value parts are lg_net_desc weights).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "lg_kernels.h"

namespace lg {

constexpr int kActNone = 2;  // identity (conv_f32_kernel treats any non-ELU, non-ReLU act as none)

// --------------------------------------------------------------- kernels

// logit[m] = bp + sum_c X[m][c] wp[c];  x361[m] = bv + sum_c X[m][c] wv[c]
__global__ void st_heads_fwd(const float *__restrict__ X, int M, int C, const float *__restrict__ wp,
                             const float *__restrict__ bp, const float *__restrict__ wv,
                             const float *__restrict__ bv, float *__restrict__ logits,
                             float *__restrict__ x361) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x % 32;
    if (warp >= M) return;
    const float *x = X + (size_t)warp * C;
    float sp = 0.0f, sv = 0.0f;
    for (int c = lane; c < C; c += 32) {
        sp = fmaf(x[c], wp[c], sp);
        sv = fmaf(x[c], wv[c], sv);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sp += __shfl_xor_sync(0xffffffffu, sp, o);
        sv += __shfl_xor_sync(0xffffffffu, sv, o);
    }
    if (lane == 0) {
        logits[warp] = sp + bp[0];
        x361[warp] = sv + bv[0];
    }
}

// Per board: hid = relu(b1 + W1 x361), v = tanh(b2 + W2 . hid).  W1 is [H][361].
__global__ void st_value_fwd(const float *__restrict__ x361, int B, int H, const float *__restrict__ W1,
                             const float *__restrict__ b1, const float *__restrict__ W2,
                             const float *__restrict__ b2, float *__restrict__ hid,
                             float *__restrict__ v) {
    __shared__ float xs[kPoints];
    __shared__ float part[32];
    const int b = blockIdx.x;
    if (b >= B) return;
    for (int i = threadIdx.x; i < kPoints; i += blockDim.x) xs[i] = x361[(size_t)b * kPoints + i];
    __syncthreads();
    float acc = 0.0f;
    for (int h = threadIdx.x; h < H; h += blockDim.x) {
        float s = b1[h];
        for (int i = 0; i < kPoints; ++i) s = fmaf(W1[(size_t)h * kPoints + i], xs[i], s);
        s = fmaxf(s, 0.0f);
        hid[(size_t)b * H + h] = s;
        acc = fmaf(W2[h], s, acc);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (threadIdx.x % 32 == 0) part[threadIdx.x / 32] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.0f;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) s += part[w];
        v[b] = tanhf(b2[0] + s);
    }
}

// softmax at temperature 1, per board (inference output of the FP32 student)
__global__ void st_softmax(const float *__restrict__ logits, int B, float *__restrict__ probs) {
    __shared__ float red[32];
    const int b = blockIdx.x, p = threadIdx.x;
    float x = p < kPoints ? logits[(size_t)b * kPoints + p] : -3.0e38f;
    float m = x;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (p % 32 == 0) red[p / 32] = m;
    __syncthreads();
    m = red[0];
    for (int w = 1; w < 12; ++w) m = fmaxf(m, red[w]);
    __syncthreads();
    float e = p < kPoints ? expf(x - m) : 0.0f;
    float s = e;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (p % 32 == 0) red[p / 32] = s;
    __syncthreads();
    s = 0.0f;
    for (int w = 0; w < 12; ++w) s += red[w];
    if (p < kPoints) probs[(size_t)b * kPoints + p] = e / s;
}

// Per board: loss and head gradients.
//   dlogits = (softmax - target) / B
//   du = 2 vw (v - vt)(1 - v^2) / B;  dpre[h] = du W2[h] [hid > 0];  dx361 = W1^T dpre
// Writes dlogits[B][361], du[B], dpre[B][H], dx361[B][361]; adds the batch
// losses into loss[0] (KL) and loss[1] (value MSE, before vw).
__global__ void __launch_bounds__(384) st_loss_bwd(const float *__restrict__ logits, const float *__restrict__ target,
                            const float *__restrict__ v, const float *__restrict__ vt,
                            const float *__restrict__ hid, const float *__restrict__ W1,
                            const float *__restrict__ W2, int B, int H, float vw,
                            float *__restrict__ dlogits, float *__restrict__ du_out,
                            float *__restrict__ dpre, float *__restrict__ dx361,
                            float *__restrict__ loss) {
    __shared__ float red[32];
    __shared__ float s_dpre[512];
    const int b = blockIdx.x, p = threadIdx.x;
    const float invB = 1.0f / (float)B;
    const float x = p < kPoints ? logits[(size_t)b * kPoints + p] : -3.0e38f;
    float m = x;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (p % 32 == 0) red[p / 32] = m;
    __syncthreads();
    m = red[0];
    for (int w = 1; w < 12; ++w) m = fmaxf(m, red[w]);
    __syncthreads();
    const float e = p < kPoints ? expf(x - m) : 0.0f;
    float s = e;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (p % 32 == 0) red[p / 32] = s;
    __syncthreads();
    s = 0.0f;
    for (int w = 0; w < 12; ++w) s += red[w];
    __syncthreads();
    float kl = 0.0f;
    if (p < kPoints) {
        const float t = target[(size_t)b * kPoints + p];
        const float logq = (x - m) - logf(s);
        dlogits[(size_t)b * kPoints + p] = (e / s - t) * invB;
        if (t > 0.0f) kl = t * (logf(t) - logq);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) kl += __shfl_xor_sync(0xffffffffu, kl, o);
    if (p % 32 == 0) red[p / 32] = kl;
    __syncthreads();
    if (p == 0) {
        float t = 0.0f;
        for (int w = 0; w < 12; ++w) t += red[w];
        atomicAdd(&loss[0], t * invB);
    }
    // value head
    const float vb = v[b], d = vb - vt[b];
    const float du = 2.0f * vw * d * (1.0f - vb * vb) * invB;
    if (p == 0) {
        du_out[b] = du;
        atomicAdd(&loss[1], d * d * invB);
    }
    for (int h = p; h < H; h += blockDim.x) {
        const float g = (hid[(size_t)b * H + h] > 0.0f) ? du * W2[h] : 0.0f;
        s_dpre[h] = g;
        dpre[(size_t)b * H + h] = g;
    }
    __syncthreads();
    if (p < kPoints) {
        float acc = 0.0f;
        for (int h = 0; h < H; ++h) acc = fmaf(s_dpre[h], W1[(size_t)h * kPoints + p], acc);
        dx361[(size_t)b * kPoints + p] = acc;
    }
}

// Value FC weight gradients, reduced over the batch (one CTA per hidden unit):
//   dW1[h][i] = sum_b dpre[b][h] x361[b][i], db1[h] = sum_b dpre[b][h],
//   dW2[h] = sum_b du[b] hid[b][h], db2 = sum_b du[b]  (CTA 0).
__global__ void st_fc_wgrad(const float *__restrict__ dpre, const float *__restrict__ du,
                            const float *__restrict__ x361, const float *__restrict__ hid, int B, int H,
                            float *__restrict__ dW1, float *__restrict__ db1, float *__restrict__ dW2,
                            float *__restrict__ db2) {
    const int h = blockIdx.x;
    for (int i = threadIdx.x; i < kPoints; i += blockDim.x) {
        float s = 0.0f;
        for (int b = 0; b < B; ++b) s = fmaf(dpre[(size_t)b * H + h], x361[(size_t)b * kPoints + i], s);
        dW1[(size_t)h * kPoints + i] += s;
    }
    if (threadIdx.x == 0) {
        float s1 = 0.0f, s2 = 0.0f;
        for (int b = 0; b < B; ++b) {
            s1 += dpre[(size_t)b * H + h];
            s2 = fmaf(du[b], hid[(size_t)b * H + h], s2);
        }
        db1[h] += s1;
        dW2[h] += s2;
    }
    if (h == 0 && threadIdx.x == 32) {
        float s = 0.0f;
        for (int b = 0; b < B; ++b) s += du[b];
        db2[0] += s;
    }
}

// Head backward into the trunk: dX[m][c] = dlogits[m] wp[c] + dx361[m] wv[c];
// head weight gradients dwp[c] = sum_m dlogits[m] X[m][c] (dwv alike),
// dbp = sum_m dlogits[m], dbv = sum_m dx361[m].  C <= 128.
__global__ void __launch_bounds__(256) st_heads_bwd(const float *__restrict__ X, const float *__restrict__ dlogits,
                             const float *__restrict__ dx361, const float *__restrict__ wp,
                             const float *__restrict__ wv, int M, int C, float *__restrict__ dX,
                             float *__restrict__ dwp, float *__restrict__ dbp,
                             float *__restrict__ dwv, float *__restrict__ dbv) {
    __shared__ float swp[128], swv[128], sdp[256][2];
    const int tid = threadIdx.x;
    // Each thread owns channel c = tid % C of rows m = row0 + tid / C + k*(256/C).
    const int per = 256 / C;
    const int c = tid % C, r = tid / C;
    float gp = 0.0f, gv = 0.0f, bpp = 0.0f, bvv = 0.0f;
    for (int m = blockIdx.x * per + r; m < M && r < per; m += gridDim.x * per) {
        const float dl = dlogits[m], dx = dx361[m];
        const float x = X[(size_t)m * C + c];
        dX[(size_t)m * C + c] = dl * wp[c] + dx * wv[c];
        gp = fmaf(dl, x, gp);
        gv = fmaf(dx, x, gv);
        if (c == 0) {
            bpp += dl;
            bvv += dx;
        }
    }
    if (tid < C) {
        swp[tid] = 0.0f;
        swv[tid] = 0.0f;
    }
    sdp[tid][0] = bpp;
    sdp[tid][1] = bvv;
    __syncthreads();
    if (r < per) {
        atomicAdd(&swp[c], gp);
        atomicAdd(&swv[c], gv);
    }
    __syncthreads();
    if (tid < C) {
        atomicAdd(&dwp[tid], swp[tid]);
        atomicAdd(&dwv[tid], swv[tid]);
    }
    if (tid == 0) {
        float a = 0.0f, b = 0.0f;
        for (int i = 0; i < 256; ++i) {
            a += sdp[i][0];
            b += sdp[i][1];
        }
        atomicAdd(dbp, a);
        atomicAdd(dbv, b);
    }
}

// dYpre = dY * (Y > 0) in place; db[o] += sum_m dYpre[m][o].  C <= 256.
__global__ void __launch_bounds__(256) st_relu_bwd(float *__restrict__ dY, const float *__restrict__ Y, int M, int C,
                            float *__restrict__ db) {
    __shared__ float sb[256];
    const int tid = threadIdx.x;
    if (tid < C) sb[tid] = 0.0f;
    __syncthreads();
    const size_t total = (size_t)M * C;
    float acc = 0.0f;
    // stride is a multiple of C (256 threads * grid, C divides 256), so each
    // thread stays on one channel
    const int c = tid % C;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + tid; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const float g = Y[i] > 0.0f ? dY[i] : 0.0f;
        dY[i] = g;
        acc += g;
    }
    atomicAdd(&sb[c], acc);
    __syncthreads();
    if (tid < C) atomicAdd(&db[tid], sb[tid]);
}

// dW[tap][c][o] += sum over rows m in this CTA's chunk of
//   X[m + shift(tap)][c] * dY[m][o]   (X zero outside the board).
// Grid: (taps, row chunks, cin tiles of 64); 256 threads, 64 x 64 output tile
// (cout <= 64 per tile pass; two passes for cout 128), 4 x 4 per thread.
template <int KS>
__global__ void __launch_bounds__(256) st_conv_wgrad(const float *__restrict__ X, const float *__restrict__ dY, int M,
                              int Cin, int Cout, int rows_per_cta, float *__restrict__ dW) {
    constexpr int PAD = KS / 2;
    __shared__ float Xs[32][65];
    __shared__ float Gs[32][65];
    const int tap = blockIdx.x;
    const int dy = tap / KS - PAD, dx = tap % KS - PAD;
    const int m0 = blockIdx.y * rows_per_cta;
    const int m1 = min(M, m0 + rows_per_cta);
    const int c0 = blockIdx.z * 64;
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    for (int o0 = 0; o0 < Cout; o0 += 64) {
        float acc[4][4] = {};
        for (int mb = m0; mb < m1; mb += 32) {
            for (int i = tid; i < 32 * 64; i += 256) {
                const int rr = i / 64, cc = i % 64;
                const int m = mb + rr;
                float xv = 0.0f, gv = 0.0f;
                if (m < m1) {
                    const int b = m / kPoints, p = m % kPoints;
                    const int y = p / kBoard + dy, x = p % kBoard + dx;
                    if (c0 + cc < Cin && y >= 0 && y < kBoard && x >= 0 && x < kBoard)
                        xv = X[((size_t)b * kPoints + y * kBoard + x) * Cin + c0 + cc];
                    if (o0 + cc < Cout) gv = dY[(size_t)m * Cout + o0 + cc];
                }
                Xs[rr][cc] = xv;
                Gs[rr][cc] = gv;
            }
            __syncthreads();
#pragma unroll 8
            for (int rr = 0; rr < 32; ++rr) {
                float a[4], g[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) a[i] = Xs[rr][ty + 16 * i];
#pragma unroll
                for (int j = 0; j < 4; ++j) g[j] = Gs[rr][tx + 16 * j];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], g[j], acc[i][j]);
            }
            __syncthreads();
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int c = c0 + ty + 16 * i;
            if (c >= Cin) continue;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int o = o0 + tx + 16 * j;
                if (o < Cout) atomicAdd(&dW[((size_t)tap * Cin + c) * Cout + o], acc[i][j]);
            }
        }
    }
}

// wtT[t'][o][c] = wt[k*k-1-t'][c][o]: the input-gradient conv's weights.
__global__ void st_flip_weights(const float *__restrict__ wt, int kk, int Cin, int Cout,
                                float *__restrict__ wtT) {
    const size_t total = (size_t)kk * Cin * Cout;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int t = (int)(i / ((size_t)Cin * Cout));
        const int rem = (int)(i % ((size_t)Cin * Cout));
        const int o = rem / Cin, c = rem % Cin;
        wtT[i] = wt[((size_t)(kk - 1 - t) * Cin + c) * Cout + o];
    }
}

__global__ void st_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                        float *__restrict__ v, size_t n, float lr, float b1, float b2, float eps,
                        float c1, float c2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

}  // namespace lg

// ====================================================================== C ABI

using namespace lg;

struct lg_student {
    int device = 0, c_in = 0, width = 0, n3x3 = 0, H = 0, max_batch = 0;
    cudaStream_t stream = nullptr;
    std::vector<void *> allocs;
    // parameter tensors (offsets into params / grads, in floats)
    struct Conv {
        int k, cin, cout;
        size_t w, b;     // GPU layout [tap][cin][cout], bias
        float *wtT;      // flipped/transposed copy for the input gradient
    };
    std::vector<Conv> convs;
    size_t wp, bp, wv, bv, W1, b1, W2, b2, nparam = 0;
    float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
    long long step = 0;
    // activations and gradients
    float *X0 = nullptr;
    std::vector<float *> Y;  // outputs of every conv (post-ReLU)
    float *logits = nullptr, *x361 = nullptr, *hid = nullptr, *vout = nullptr;
    float *dA = nullptr, *dB = nullptr, *dlogits = nullptr, *dx361 = nullptr, *dpre = nullptr,
          *du = nullptr, *partial = nullptr, *zeros = nullptr, *loss = nullptr;
    std::mutex mu;
};

namespace {

template <class T>
int st_alloc(lg_student *s, T **p, size_t count) {
    if (cudaMalloc((void **)p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) {
        lg_set_error("cudaMalloc failed (%zu bytes)", count * sizeof(T));
        return LG_ERR_ALLOC;
    }
    s->allocs.push_back(*p);
    return LG_OK;
}

float *P(lg_student *s, size_t off) { return s->params + off; }
float *G(lg_student *s, size_t off) { return s->grads + off; }

// Forward in FP32, saving every activation.  planes: device [B][c_in][361].
int st_forward(lg_student *s, const uint8_t *planes, int B, cudaStream_t st) {
    const int M = B * kPoints;
    launch_pack_planes_f32(planes, B, s->c_in, s->X0, st);
    const float *in = s->X0;
    for (size_t l = 0; l < s->convs.size(); ++l) {
        auto &c = s->convs[l];
        launch_conv_f32(in, P(s, c.w), P(s, c.b), s->Y[l], B, c.cin, c.cout, c.k, LG_ACT_RELU, s->partial, st);
        in = s->Y[l];
    }
    st_heads_fwd<<<(M * 32 + 255) / 256, 256, 0, st>>>(in, M, s->width, P(s, s->wp), P(s, s->bp),
                                                       P(s, s->wv), P(s, s->bv), s->logits, s->x361);
    st_value_fwd<<<B, 64, 0, st>>>(s->x361, B, s->H, P(s, s->W1), P(s, s->b1), P(s, s->W2), P(s, s->b2),
                                   s->hid, s->vout);
    return LG_OK;
}

int st_backward(lg_student *s, int B, const float *target, const float *vt, float vw, cudaStream_t st) {
    const int M = B * kPoints;
    cudaMemsetAsync(s->grads, 0, s->nparam * sizeof(float), st);
    cudaMemsetAsync(s->loss, 0, 2 * sizeof(float), st);
    st_loss_bwd<<<B, 384, 0, st>>>(s->logits, target, s->vout, vt, s->hid, P(s, s->W1), P(s, s->W2), B, s->H,
                                   vw, s->dlogits, s->du, s->dpre, s->dx361, s->loss);
    st_fc_wgrad<<<s->H, 128, 0, st>>>(s->dpre, s->du, s->x361, s->hid, B, s->H, G(s, s->W1), G(s, s->b1),
                                      G(s, s->W2), G(s, s->b2));
    const float *Xlast = s->Y.back();
    int hblocks = std::min(1024, (M + (256 / s->width) - 1) / (256 / s->width));
    st_heads_bwd<<<hblocks, 256, 0, st>>>(Xlast, s->dlogits, s->dx361, P(s, s->wp), P(s, s->wv), M, s->width,
                                          s->dA, G(s, s->wp), G(s, s->bp), G(s, s->wv), G(s, s->bv));
    float *dY = s->dA, *dX = s->dB;
    for (int l = (int)s->convs.size() - 1; l >= 0; --l) {
        auto &c = s->convs[l];
        const float *Xin = l > 0 ? s->Y[l - 1] : s->X0;
        int rblocks = std::min(1024, (int)(((size_t)M * c.cout + 255) / 256));
        st_relu_bwd<<<rblocks, 256, 0, st>>>(dY, s->Y[l], M, c.cout, G(s, c.b));
        const int rows_per_cta = 2048;
        dim3 wg(c.k * c.k, (M + rows_per_cta - 1) / rows_per_cta, (c.cin + 63) / 64);
        if (c.k == 5)
            st_conv_wgrad<5><<<wg, 256, 0, st>>>(Xin, dY, M, c.cin, c.cout, rows_per_cta, G(s, c.w));
        else if (c.k == 3)
            st_conv_wgrad<3><<<wg, 256, 0, st>>>(Xin, dY, M, c.cin, c.cout, rows_per_cta, G(s, c.w));
        else
            st_conv_wgrad<1><<<wg, 256, 0, st>>>(Xin, dY, M, c.cin, c.cout, rows_per_cta, G(s, c.w));
        if (l > 0) {
            st_flip_weights<<<64, 256, 0, st>>>(P(s, c.w), c.k * c.k, c.cin, c.cout, c.wtT);
            launch_conv_f32(dY, c.wtT, s->zeros, dX, B, c.cout, c.cin, c.k, kActNone, s->partial, st);
            std::swap(dY, dX);
        }
    }
    return LG_OK;
}

bool valid_batch(lg_student *s, int B) { return s && B >= 1 && B <= s->max_batch; }

}  // namespace

extern "C" void lg_student_destroy(lg_student *s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (void *p : s->allocs) cudaFree(p);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

extern "C" int lg_student_create(int device, int c_in, int width, int n3x3, int fc_hidden, int max_batch,
                                 lg_student **out) {
    if (!out || c_in < 1 || c_in > 64 || width < 16 || width > 128 || (256 % width) != 0 || n3x3 < 0 ||
        n3x3 > 32 || fc_hidden < 1 || fc_hidden > 512 || max_batch < 1 || max_batch > 4096) {
        lg_set_error("lg_student_create: bad arguments (width must divide 256)");
        return LG_ERR_ARG;
    }
    *out = nullptr;
    lg_student *s = new lg_student();
    s->device = device;
    s->c_in = c_in;
    s->width = width;
    s->n3x3 = n3x3;
    s->H = fc_hidden;
    s->max_batch = max_batch;
    auto fail = [&](int rc) {
        lg_student_destroy(s);
        return rc;
    };
    if (cudaSetDevice(device) != cudaSuccess) {
        lg_set_error("no CUDA device %d", device);
        return fail(LG_ERR_CUDA);
    }
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(LG_ERR_CUDA);
    size_t off = 0;
    for (int l = 0; l <= n3x3; ++l) {
        lg_student::Conv c{};
        c.k = l == 0 ? 5 : 3;
        c.cin = l == 0 ? c_in : width;
        c.cout = width;
        c.w = off;
        off += (size_t)c.k * c.k * c.cin * c.cout;
        c.b = off;
        off += c.cout;
        s->convs.push_back(c);
    }
    s->wp = off; off += width;
    s->bp = off; off += 1;
    s->wv = off; off += width;
    s->bv = off; off += 1;
    s->W1 = off; off += (size_t)fc_hidden * kPoints;
    s->b1 = off; off += fc_hidden;
    s->W2 = off; off += fc_hidden;
    s->b2 = off; off += 1;
    s->nparam = off;
    const size_t M = (size_t)max_batch * kPoints;
    int rc;
    if ((rc = st_alloc(s, &s->params, off)) || (rc = st_alloc(s, &s->grads, off)) ||
        (rc = st_alloc(s, &s->m, off)) || (rc = st_alloc(s, &s->v, off)) ||
        (rc = st_alloc(s, &s->X0, M * c_in)) || (rc = st_alloc(s, &s->logits, M)) ||
        (rc = st_alloc(s, &s->x361, M)) || (rc = st_alloc(s, &s->hid, (size_t)max_batch * fc_hidden)) ||
        (rc = st_alloc(s, &s->vout, max_batch)) || (rc = st_alloc(s, &s->dA, M * width)) ||
        (rc = st_alloc(s, &s->dB, M * width)) || (rc = st_alloc(s, &s->dlogits, M)) ||
        (rc = st_alloc(s, &s->dx361, M)) || (rc = st_alloc(s, &s->dpre, (size_t)max_batch * fc_hidden)) ||
        (rc = st_alloc(s, &s->du, max_batch)) || (rc = st_alloc(s, &s->zeros, 256)) ||
        (rc = st_alloc(s, &s->loss, 2)))
        return fail(rc);
    size_t maxpart = 0;
    for (int b = 1; b <= max_batch; b = b < 64 ? b + 1 : b * 2)
        for (auto &c : s->convs) {
            maxpart = std::max(maxpart, conv_f32_partial_floats(b, c.cin, c.cout, c.k));
            maxpart = std::max(maxpart, conv_f32_partial_floats(b, c.cout, c.cin, c.k));
        }
    if ((rc = st_alloc(s, &s->partial, maxpart))) return fail(rc);
    for (auto &c : s->convs) {
        float *y;
        if ((rc = st_alloc(s, &y, M * width))) return fail(rc);
        s->Y.push_back(y);
        if ((rc = st_alloc(s, &c.wtT, (size_t)c.k * c.k * c.cin * c.cout))) return fail(rc);
    }
    cudaMemset(s->zeros, 0, 256 * sizeof(float));
    cudaMemset(s->params, 0, off * sizeof(float));
    cudaMemset(s->m, 0, off * sizeof(float));
    cudaMemset(s->v, 0, off * sizeof(float));
    if (cudaDeviceSynchronize() != cudaSuccess) return fail(LG_ERR_CUDA);
    *out = s;
    return LG_OK;
}

extern "C" size_t lg_student_param_count(const lg_student *s) { return s ? s->nparam : 0; }

// Host flat layout (OIHW per conv, then the heads and FCs) <-> GPU layout.
extern "C" int lg_student_set_params(lg_student *s, const float *host, size_t n) {
    if (!s || !host || n != s->nparam) {
        lg_set_error("lg_student_set_params: expected %zu floats", s ? s->nparam : 0);
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(s->mu);
    std::vector<float> gpu(n);
    size_t hoff = 0;
    for (auto &c : s->convs) {
        const int kk = c.k * c.k;
        for (int o = 0; o < c.cout; ++o)
            for (int ci = 0; ci < c.cin; ++ci)
                for (int t = 0; t < kk; ++t)
                    gpu[c.w + ((size_t)t * c.cin + ci) * c.cout + o] = host[hoff + ((size_t)o * c.cin + ci) * kk + t];
        hoff += (size_t)kk * c.cin * c.cout;
        std::memcpy(&gpu[c.b], host + hoff, c.cout * sizeof(float));
        hoff += c.cout;
    }
    std::memcpy(&gpu[s->wp], host + hoff, (n - hoff) * sizeof(float));  // heads + FC: same order
    cudaSetDevice(s->device);
    LG_CUDA_TRY(cudaMemcpy(s->params, gpu.data(), n * sizeof(float), cudaMemcpyHostToDevice));
    LG_CUDA_TRY(cudaMemset(s->m, 0, n * sizeof(float)));
    LG_CUDA_TRY(cudaMemset(s->v, 0, n * sizeof(float)));
    s->step = 0;
    return LG_OK;
}

static int to_host_layout(lg_student *s, const float *dev, float *host) {
    std::vector<float> gpu(s->nparam);
    LG_CUDA_TRY(cudaMemcpy(gpu.data(), dev, s->nparam * sizeof(float), cudaMemcpyDeviceToHost));
    size_t hoff = 0;
    for (auto &c : s->convs) {
        const int kk = c.k * c.k;
        for (int o = 0; o < c.cout; ++o)
            for (int ci = 0; ci < c.cin; ++ci)
                for (int t = 0; t < kk; ++t)
                    host[hoff + ((size_t)o * c.cin + ci) * kk + t] = gpu[c.w + ((size_t)t * c.cin + ci) * c.cout + o];
        hoff += (size_t)kk * c.cin * c.cout;
        std::memcpy(host + hoff, &gpu[c.b], c.cout * sizeof(float));
        hoff += c.cout;
    }
    std::memcpy(host + hoff, &gpu[s->wp], (s->nparam - hoff) * sizeof(float));
    return LG_OK;
}

extern "C" int lg_student_get_params(lg_student *s, float *host, size_t n) {
    if (!s || !host || n != s->nparam) {
        lg_set_error("lg_student_get_params: expected %zu floats", s ? s->nparam : 0);
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(s->mu);
    cudaSetDevice(s->device);
    return to_host_layout(s, s->params, host);
}

extern "C" int lg_student_grads(lg_student *s, const uint8_t *planes, int B, const float *target_probs,
                                const float *target_value, float value_weight, float *host_grads,
                                float *host_loss) {
    if (!valid_batch(s, B) || !planes || !target_probs || !target_value || !host_grads) {
        lg_set_error("lg_student_grads: bad arguments");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(s->mu);
    cudaSetDevice(s->device);
    st_forward(s, planes, B, s->stream);
    st_backward(s, B, target_probs, target_value, value_weight, s->stream);
    LG_CUDA_TRY(cudaGetLastError());
    LG_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (host_loss) LG_CUDA_TRY(cudaMemcpy(host_loss, s->loss, 2 * sizeof(float), cudaMemcpyDeviceToHost));
    return to_host_layout(s, s->grads, host_grads);
}

extern "C" int lg_student_train_step(lg_student *s, const uint8_t *planes, int B, const float *target_probs,
                                     const float *target_value, float lr, float value_weight, float *host_loss,
                                     void *stream) {
    if (!valid_batch(s, B) || !planes || !target_probs || !target_value || !(lr > 0.0f)) {
        lg_set_error("lg_student_train_step: bad arguments");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(s->mu);
    cudaSetDevice(s->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    st_forward(s, planes, B, st);
    st_backward(s, B, target_probs, target_value, value_weight, st);
    s->step += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, (float)s->step), c2 = 1.0f - std::pow(b2, (float)s->step);
    st_adam<<<512, 256, 0, st>>>(s->params, s->grads, s->m, s->v, s->nparam, lr, b1, b2, 1e-8f, c1, c2);
    LG_CUDA_TRY(cudaGetLastError());
    if (host_loss) {
        LG_CUDA_TRY(cudaMemcpyAsync(host_loss, s->loss, 2 * sizeof(float), cudaMemcpyDeviceToHost, st));
        LG_CUDA_TRY(cudaStreamSynchronize(st));
    }
    return LG_OK;
}

extern "C" int lg_student_forward(lg_student *s, const uint8_t *planes, int B, float *probs, float *value,
                                  void *stream) {
    if (!valid_batch(s, B) || !planes || !probs || !value) {
        lg_set_error("lg_student_forward: bad arguments");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(s->mu);
    cudaSetDevice(s->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    st_forward(s, planes, B, st);
    st_softmax<<<B, 384, 0, st>>>(s->logits, B, probs);
    LG_CUDA_TRY(cudaMemcpyAsync(value, s->vout, B * sizeof(float), cudaMemcpyDeviceToDevice, st));
    LG_CUDA_TRY(cudaGetLastError());
    return LG_OK;
}

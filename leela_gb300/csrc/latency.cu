// latency.cu -- small-batch forward: every layer of a net in one cooperative
// launch, for the 1..8 positions a search thread evaluates at a time.
//
// Reference: the per-leaf calls of the engine are batch 1
// (Network::get_scored_moves_internal / get_value_internal,
// Network.cpp:676-832; OpenCL_Network::forward, OpenCL.cpp:490-569, launches
// 26 kernels and a blocking finish per position).  At batch 1 a 3x3 128->128
// layer is 53 M multiply-adds -- about 1.3 us of the whole GPU's FP32 rate --
// so a launch per layer, or a GEMM tile shape made for large batches, leaves
// most of the time to launch gaps and idle SMs.
//
// Here one launch runs the whole net.  Each conv layer (the head included,
// as a layer of one output channel) is cut into units (board row (b, y),
// input-channel split s): a unit computes the layer's partial sums over the
// s-th eighth of the input channels for the 19 points of one board row and
// all output channels, and stores them (FP32) in part[layer & 1][s][b*19+y].
// The consumer of a row (the next layer's units, or the finish stage) adds
// the 8 partial sums in a fixed order, then the producing layer's scale,
// bias and activation, while it stages its input -- so no layer needs a
// reduction pass of its own and the result does not depend on scheduling.
//
// CTA c (grid G, a multiple of 8, one CTA per SM) always takes split
// s = c % 8 and rows c/8, c/8 + G/8, ...; its weight slice of a layer is one
// contiguous block, copied into shared memory with cp.async while the
// previous layer computes.  Units publish "row done" by a release add on a
// per-(layer, row) counter; a unit waits (bounded acquire polls) until the
// rows its taps read are complete in the layer before -- and, so that it
// never overwrites partial sums that are still being read, until the rows
// that read the same rows of the layer before it are complete.  No
// grid-wide barrier; the last CTA to leave resets the counters for the next
// launch.
//
// Arithmetic per thread: 5 points x 2 output channels, the 5 + k - 1 input
// values of one (channel, tap row) read once into registers (every lane of
// a warp reads the same ones: a shared-memory broadcast), the weights as
// float2 (consecutive lanes, consecutive channels).  Partial sums are read
// with ld.global.cg (L2, never a stale L1 line from an earlier layer).
#include "lg_kernels.h"

#include <cuda_fp16.h>

#include <algorithm>
#include <cfloat>

namespace lg {

namespace {

constexpr int kLT = 256;                       // threads per CTA
constexpr int kRowPts = 20;                    // 19 points + one pad column
constexpr int kPitch = 24;                     // staged input row: x = -r .. 19 + r
constexpr uint32_t kLatPolls = 1u << 22;       // default limit, x ~32-64 ns: bounded at ~0.3 s
constexpr size_t kPartBuf = (size_t)kLatSplits * kLatMaxRows * kRowPts * 128;  // floats per parity

__device__ __forceinline__ float lat_act(float v, int act) {
    if (act == LG_ACT_ELU) return (v > 0.0f) ? v : (expf(v) - 1.0f);
    return fmaxf(v, 0.0f);
}

__device__ __forceinline__ int ld_acq(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_release_add(int *p, int v) {
    asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int atom_acq_rel_add(int *p, int v) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(ptx::smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Polls one counter until it reaches `want`: spins, then sleeps between
// polls; gives up after `limit` polls or as soon as another CTA has
// reported an error.  Returns false on either.
__device__ __forceinline__ bool poll_one(const int *c, int want, const int *err, uint32_t limit) {
    uint32_t n = 0;
    while (ld_acq(c) < want) {
        if (++n >= limit || *(volatile const int *)err != 0) return false;
        if (n > 64) __nanosleep(32);
    }
    return true;
}

// The CTA waits until counters cnt[lo..hi] (hi - lo < kLT) reach `want`,
// one polling thread per counter; true for every thread if all did.
__device__ __forceinline__ bool wait_rows(const int *cnt, int lo, int hi, int want, const int *err, bool alive,
                                          uint32_t limit) {
    const int t = threadIdx.x;
    const bool bad = t <= hi - lo && alive && !poll_one(cnt + lo + t, want, err, limit);
    return !__syncthreads_or(bad || !alive);
}

// The weight slice of split s of layer L into shared memory (cp.async, 16 B
// per copy; slices are padded to 4 floats so every copy is aligned).
__device__ __forceinline__ void copy_slice(const LatConv &L, int s, float *dst) {
    const float *src = static_cast<const float *>(L.w) + (size_t)s * L.slice;
    for (int i = threadIdx.x * 4; i < L.slice; i += kLT * 4) cp_async16(dst + i, src + i);
}

// Partial sums of one unit: acc[j][h] for point 5 pg + j and channel
// 2 cp + h, over the unit's cg input channels and the K x K taps.
template <int K>
__device__ __forceinline__ void unit_mac(const float *in_s, const float *w_s, int cg, int cout, int pg, int cp,
                                         float (&acc)[5][2]) {
    const bool one = cout == 1;
    for (int c = 0; c < cg; ++c) {
#pragma unroll
        for (int dy = 0; dy < K; ++dy) {
            const float *row = in_s + (c * K + dy) * kPitch + 5 * pg;
            float iv[5 + K - 1];
#pragma unroll
            for (int i = 0; i < 5 + K - 1; ++i) iv[i] = row[i];
#pragma unroll
            for (int dx = 0; dx < K; ++dx) {
                const int widx = (c * K * K + dy * K + dx) * cout + 2 * cp;
                const float2 w = one ? make_float2(w_s[widx], 0.0f) : *reinterpret_cast<const float2 *>(w_s + widx);
#pragma unroll
                for (int j = 0; j < 5; ++j) {
                    acc[j][0] = fmaf(iv[j + dx], w.x, acc[j][0]);
                    acc[j][1] = fmaf(iv[j + dx], w.y, acc[j][1]);
                }
            }
        }
    }
}

// 16-bit layers (3x3, 16 input channels a split, 128 output channels) on
// the warp-level tensor-core MMA m16n8k16 (FP32 accumulate): warp w owns
// output channels 16 w .. 16 w + 15 (A = weights, w16[tap][o][16]), the
// three 8-point column tiles of the row (B = staged inputs,
// in16[dy][xx][16], point x at xx = x + dx), one K step of 16 channels per
// tap.  acc[j] is the accumulator fragment of column tile j: channel
// 16 w + g (+ 8 for acc[j][2..3]), points 8 j + 2 t, + 1 (g = lane / 4,
// t = lane % 4).
template <bool F16>
__device__ __forceinline__ void unit_mma(const uint16_t *in16, const uint16_t *w16, int nx, int warp, int lane,
                                         float (&acc)[3][4]) {
    const int r8 = lane & 7, mi = lane >> 3;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const int dy = t / 3, dx = t % 3;
        uint32_t a[4];
        const uint16_t *ap = w16 + (size_t)((t * 128 + 16 * warp + r8 + 8 * (mi & 1)) * 16 + 8 * (mi >> 1));
        asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                     : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3])
                     : "r"(ptx::smem_u32(ap)));
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            uint32_t b[2];
            const uint16_t *bp = in16 + (size_t)((dy * nx + 8 * j + r8 + dx) * 16 + 8 * (mi & 1));
            asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];"
                         : "=r"(b[0]), "=r"(b[1])
                         : "r"(ptx::smem_u32(bp)));
            if (F16)
                asm volatile(
                    "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                    "{%0,%1,%2,%3};"
                    : "+f"(acc[j][0]), "+f"(acc[j][1]), "+f"(acc[j][2]), "+f"(acc[j][3])
                    : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
            else
                asm volatile(
                    "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                    "{%0,%1,%2,%3};"
                    : "+f"(acc[j][0]), "+f"(acc[j][1]), "+f"(acc[j][2]), "+f"(acc[j][3])
                    : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
        }
    }
}

__device__ __forceinline__ uint16_t to16(float v, bool f16) {
    return f16 ? __half_as_ushort(__float2half_rn(v)) : __bfloat16_as_ushort(__float2bfloat16_rn(v));
}

}  // namespace

// MODE 0: FP32 throughout.  MODE 1 / 2: the layers marked `mma` take 16-bit
// inputs (BF16 / FP16, rounded as the consumer stages them) on the warp
// MMA; the first layer and the head stay FP32 FFMA on the 16-bit-rounded
// weights (as the tensor-core trunk keeps the head in FP32).
template <int MODE>
__global__ void __launch_bounds__(kLT, 1) lat_kernel(const LatParams p) {
    constexpr bool F16 = MODE == 2;
    extern __shared__ float4 lat_smem4[];
    float *sm = reinterpret_cast<float *>(lat_smem4);
    float *wbuf0 = sm, *wbuf1 = sm + kLatSliceMax;
    float *in_s = sm + 2 * kLatSliceMax;                      // [cg][K][kPitch] FP32, or in16 [K][nx][16]
    uint16_t *in16 = reinterpret_cast<uint16_t *>(in_s);
    float *fin = in_s + kLatMaxCg * 5 * kPitch;                // finish stage: 361 head outputs + 8 x 32 sums
    __shared__ int s_last;
    __shared__ float red[32];

    const int tid = threadIdx.x, G = gridDim.x, cta = blockIdx.x, lane = tid & 31, warp = tid >> 5;
    const int s = cta % kLatSplits, rstep = G / kLatSplits;
    const int rows = p.B * kBoard;
    const int cp = tid % 64, pg = tid / 64;
    bool alive = true;
    auto fail = [&](int code) {
        if (tid == 0 && alive) atomicCAS(p.err, 0, code);
        alive = false;
    };

    copy_slice(p.L[0], s, wbuf0);
    cp_async_commit();
    for (int l = 0; l < p.nl; ++l) {
        const LatConv &L = p.L[l];
        const bool mma = MODE != 0 && L.mma;
        float *w_s = (l & 1) ? wbuf1 : wbuf0;
        __syncthreads();  // the other buffer's last reader (layer l - 1) is done
        if (l + 1 < p.nl) copy_slice(p.L[l + 1], s, (l & 1) ? wbuf0 : wbuf1);
        cp_async_commit();
        cp_async_wait1();
        __syncthreads();
        const int r = L.k / 2;
        const int rp = l > 0 ? p.L[l - 1].k / 2 : 0;
        const int rw = max(r, rp);                             // rows to wait for
        const float *src = p.part + (size_t)((l - 1) & 1) * kPartBuf;
        float *dst = p.part + (size_t)(l & 1) * kPartBuf;
        // staged columns: x = -r .. 19 + r (FFMA: 20 points), or .. 23 + r
        // (MMA: three 8-point column tiles)
        const int nx = (mma ? 24 : kRowPts) + 2 * r;
        for (int row = cta / kLatSplits; row < rows; row += rstep) {
            const int b = row / kBoard, y = row % kBoard;
            // (test hook: the stalled row of layer 1 waits for a count no
            // unit reaches)
            const int want = (l == 1 && row == p.stall_row) ? kLatSplits + (1 << 20) : kLatSplits;
            if (l > 0 && !wait_rows(p.cnt + (l - 1) * kLatMaxRows, b * kBoard + max(0, y - rw),
                                    b * kBoard + min(kBoard - 1, y + rw), want, p.err, alive, p.poll_limit)) {
                fail(91);
                continue;
            }
            if (!alive) continue;
            // ---- stage the input rows y - r .. y + r of this split's channels
            const int c0 = s * L.cg;
            if (l == 0) {
                const int n = L.cg * L.k * nx;
                for (int i = tid; i < n; i += kLT) {
                    const int c = i / (L.k * nx), rem = i - c * (L.k * nx), dy = rem / nx, xx = rem - dy * nx;
                    const int yy = y + dy - r, x = xx - r;
                    float v = 0.0f;
                    if (yy >= 0 && yy < kBoard && x >= 0 && x < kBoard)
                        v = (float)p.planes[((size_t)b * p.c_in + c0 + c) * kPoints + yy * kBoard + x];
                    in_s[(c * L.k + dy) * kPitch + xx] = v;
                }
            } else {
                // 8 channels per item (4 when cg is not a multiple of 8): sum
                // of the 8 partials, scale, bias, act; every load of an item
                // is issued before the first add, and at most two items a
                // thread for a 3x3 layer (one round trip each)
                const LatConv &P = p.L[l - 1];
                const int cw = (L.cg % 8 == 0) ? 8 : 4, nc = L.cg / cw, n = nc * L.k * nx;
                for (int i = tid; i < n; i += kLT) {
                    const int ci = i / (L.k * nx), rem = i - ci * (L.k * nx), dy = rem / nx, xx = rem - dy * nx;
                    const int yy = y + dy - r, x = xx - r;
                    float v[8];
#pragma unroll
                    for (int e = 0; e < 8; ++e) v[e] = 0.0f;
                    const int ch = c0 + cw * ci;
                    if (yy >= 0 && yy < kBoard && x >= 0 && x < kBoard) {
                        const float *q = src + ((size_t)(b * kBoard + yy) * kRowPts + x) * 128 + ch;
                        float4 t[kLatSplits][2];
#pragma unroll
                        for (int ss = 0; ss < kLatSplits; ++ss) {
                            const float4 *qq = reinterpret_cast<const float4 *>(q + (size_t)ss * kLatMaxRows * kRowPts * 128);
                            t[ss][0] = __ldcg(qq);
                            t[ss][1] = cw == 8 ? __ldcg(qq + 1) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        }
#pragma unroll
                        for (int ss = 0; ss < kLatSplits; ++ss) {
                            v[0] += t[ss][0].x;
                            v[1] += t[ss][0].y;
                            v[2] += t[ss][0].z;
                            v[3] += t[ss][0].w;
                            v[4] += t[ss][1].x;
                            v[5] += t[ss][1].y;
                            v[6] += t[ss][1].z;
                            v[7] += t[ss][1].w;
                        }
#pragma unroll
                        for (int e = 0; e < 8; ++e) {
                            if (e >= cw) break;
                            const float bb = __ldg(P.bias + ch + e);
                            v[e] = lat_act(P.scale ? fmaf(v[e], __ldg(P.scale + ch + e), bb) : v[e] + bb, p.act);
                        }
                    }
                    if (mma) {
                        // cw == 8 (cg = 16): one 16-byte store of 8 channels
                        uint4 h;
                        h.x = (uint32_t)to16(v[0], F16) | ((uint32_t)to16(v[1], F16) << 16);
                        h.y = (uint32_t)to16(v[2], F16) | ((uint32_t)to16(v[3], F16) << 16);
                        h.z = (uint32_t)to16(v[4], F16) | ((uint32_t)to16(v[5], F16) << 16);
                        h.w = (uint32_t)to16(v[6], F16) | ((uint32_t)to16(v[7], F16) << 16);
                        *reinterpret_cast<uint4 *>(in16 + (dy * nx + xx) * 16 + 8 * ci) = h;
                    } else {
                        float *d = in_s + ((cw * ci) * L.k + dy) * kPitch + xx;
#pragma unroll
                        for (int e = 0; e < 8; ++e)
                            if (e < cw) d[e * L.k * kPitch] = v[e];
                    }
                }
            }
            __syncthreads();
            // ---- partial sums of this unit
            float *o_row = dst + ((size_t)s * kLatMaxRows + row) * kRowPts * 128;
            if (mma) {
                float acc[3][4];
#pragma unroll
                for (int j = 0; j < 3; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
                unit_mma<F16>(in16, reinterpret_cast<const uint16_t *>(w_s), nx, warp, lane, acc);
                const int g = lane >> 2, t4 = lane & 3, o = 16 * warp + g;
#pragma unroll
                for (int j = 0; j < 3; ++j)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int x = 8 * j + 2 * t4 + h;
                        if (x < kBoard) {
                            o_row[x * 128 + o] = acc[j][h];
                            o_row[x * 128 + o + 8] = acc[j][2 + h];
                        }
                    }
            } else if (2 * cp < L.cout) {
                float acc[5][2];
#pragma unroll
                for (int j = 0; j < 5; ++j) acc[j][0] = acc[j][1] = 0.0f;
                if (L.k == 3)
                    unit_mac<3>(in_s, w_s, L.cg, L.cout, pg, cp, acc);
                else if (L.k == 5)
                    unit_mac<5>(in_s, w_s, L.cg, L.cout, pg, cp, acc);
                else
                    unit_mac<1>(in_s, w_s, L.cg, L.cout, pg, cp, acc);
                float *o = o_row + 2 * cp;
#pragma unroll
                for (int j = 0; j < 5; ++j) {
                    const int x = 5 * pg + j;
                    if (x >= kBoard) continue;
                    if (L.cout == 1)
                        o[x * 128] = acc[j][0];
                    else
                        *reinterpret_cast<float2 *>(o + x * 128) = make_float2(acc[j][0], acc[j][1]);
                }
            }
            // publish: the barrier orders every thread's stores before thread
            // 0's release add
            __syncthreads();
            if (tid == 0) red_release_add(p.cnt + l * kLatMaxRows + row, 1);
        }
    }
    cp_async_wait0();

    // ---- finish: softmax (one unit per board) or the value head (8 units
    // per board: a slice of the FC1 units each; the last to finish adds the
    // 8 partial values in order)
    const int hl = p.nl - 1;
    const float *hsrc = p.part + (size_t)(hl & 1) * kPartBuf;
    const int nfin = p.value_head ? kLatSplits * p.B : p.B;
    for (int u = cta; u < nfin; u += G) {
        const int b = p.value_head ? u / kLatSplits : u, fs = p.value_head ? u % kLatSplits : 0;
        __syncthreads();
        if (!wait_rows(p.cnt + hl * kLatMaxRows, b * kBoard, b * kBoard + kBoard - 1, kLatSplits, p.err, alive,
                       p.poll_limit)) {
            fail(92);
            continue;
        }
        for (int i = tid; i < kPoints; i += kLT) {
            const int y = i / kBoard, x = i % kBoard;
            const float *q = hsrc + ((size_t)(b * kBoard + y) * kRowPts + x) * 128;
            float v = 0.0f;
#pragma unroll
            for (int ss = 0; ss < kLatSplits; ++ss) v += __ldcg(q + (size_t)ss * kLatMaxRows * kRowPts * 128);
            v += p.head_b;
            if (p.act_head) v = lat_act(v, p.act);
            fin[i] = v;
            if (p.logits_out && fs == 0) p.logits_out[(size_t)b * kPoints + i] = v;
        }
        __syncthreads();
        if (!p.value_head) {
            // Network.cpp:450-469: alpha = max / T; p = exp(x / T - alpha) / sum
            float m = -FLT_MAX;
            for (int i = tid; i < kPoints; i += kLT) m = fmaxf(m, fin[i]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane == 0) red[warp] = m;
            __syncthreads();
            if (tid < 32) {
                float v = tid < kLT / 32 ? red[tid] : -FLT_MAX;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
                if (tid == 0) red[16] = v;
            }
            __syncthreads();
            const float alpha = red[16] / p.temperature;
            float e[2] = {0.0f, 0.0f}, sum = 0.0f;
            for (int k = 0, i = tid; i < kPoints; i += kLT, ++k) {
                e[k] = expf(fin[i] / p.temperature - alpha);
                sum += e[k];
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
            __syncthreads();
            if (lane == 0) red[warp] = sum;
            __syncthreads();
            if (tid < 32) {
                float v = tid < kLT / 32 ? red[tid] : 0.0f;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                if (tid == 0) red[17] = v;
            }
            __syncthreads();
            const float den = red[17];
            for (int k = 0, i = tid; i < kPoints; i += kLT, ++k) p.probs[(size_t)b * kPoints + i] = e[k] / den;
        } else {
            // FC1 units fs * hs .. + hs (hs = H / 8 <= 32): lane = unit, the 8
            // warps take 8 ranges of the 361 inputs, summed in warp order
            const int hs = p.H / kLatSplits;
            const int u0 = fs * hs + lane;
            const int i0 = warp * 46, i1 = min(kPoints, i0 + 46);
            float a = 0.0f;
            if (lane < hs)
                for (int i = i0; i < i1; ++i)
                    a = fmaf(fin[i], p.w1s[((size_t)(u0 / 64) * kPoints + i) * 64 + u0 % 64], a);
            float *fs_sum = fin + 384;
            fs_sum[warp * 32 + lane] = a;
            __syncthreads();
            if (warp == 0) {
                float z = 0.0f;
                if (lane < hs) {
                    z = p.b1[u0];
                    for (int w = 0; w < kLT / 32; ++w) z += fs_sum[w * 32 + lane];
                    z = p.w2[u0] * lat_act(z, p.act);
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) z += __shfl_xor_sync(0xffffffffu, z, o);
                if (lane == 0) {
                    p.fcv[b * kLatSplits + fs] = z;
                    __threadfence();
                    const int old = atom_acq_rel_add(p.cnt + kLatCntFc + b, 1);
                    if (old == kLatSplits - 1) {
                        float x = p.b2;
                        for (int k = 0; k < kLatSplits; ++k) x += *(volatile float *)(p.fcv + b * kLatSplits + k);
                        const float t = tanhf(x);
                        p.value[b] = p.value_map == 2 ? x : (p.value_map ? (1.0f + t) / 2.0f : t);
                    }
                }
            }
        }
    }

    // ---- leave: the last CTA resets the counters for the next launch
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        s_last = atom_acq_rel_add(p.cnt + kLatCntExit, 1) == G - 1;
    }
    __syncthreads();
    if (s_last) {
        for (int i = tid; i < kLatCntExit; i += kLT) p.cnt[i] = 0;
        __syncthreads();
        if (tid == 0) p.cnt[kLatCntExit] = 0;
    }
}

size_t lat_part_floats() { return 2 * kPartBuf; }

size_t lat_smem_bytes() {
    return (size_t)(2 * kLatSliceMax + kLatMaxCg * 5 * kPitch + 384 + 8 * 32) * sizeof(float);
}

int lat_init_device() {
    cudaError_t e = cudaFuncSetAttribute(lat_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)lat_smem_bytes());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(lat_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lat_smem_bytes());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(lat_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lat_smem_bytes());
    if (e != cudaSuccess) {
        lg_set_error("cudaFuncSetAttribute(latency kernel): %s", cudaGetErrorString(e));
        return LG_ERR_CUDA;
    }
    return LG_OK;
}

int lat_grid(int B, int sm_count) {
    int g = std::min(sm_count, kLatSplits * B * kBoard);
    return g - g % kLatSplits;
}

int launch_lat(const LatParams &p_in, int mode, int sm_count, cudaStream_t s) {
    LatParams p = p_in;
    if (!p.poll_limit) p.poll_limit = kLatPolls;
    const int G = lat_grid(p.B, sm_count);
    if (p.B < 1 || p.B > kLatMaxB || p.nl < 2 || p.nl > kLatMaxLayers || G < kLatSplits || mode < 0 || mode > 2) {
        lg_set_error("latency kernel: bad arguments (B=%d, layers=%d)", p.B, p.nl);
        return LG_ERR_ARG;
    }
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(G);
    cfg.blockDim = dim3(kLT);
    cfg.dynamicSmemBytes = lat_smem_bytes();
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = mode == 0 ? cudaLaunchKernelEx(&cfg, lat_kernel<0>, p)
                              : (mode == 1 ? cudaLaunchKernelEx(&cfg, lat_kernel<1>, p)
                                           : cudaLaunchKernelEx(&cfg, lat_kernel<2>, p));
    if (e != cudaSuccess) {
        lg_set_error("latency kernel launch: %s", cudaGetErrorString(e));
        return LG_ERR_CUDA;
    }
    return LG_OK;
}

}  // namespace lg

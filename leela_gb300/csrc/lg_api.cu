// lg_api.cu -- the C ABI (include/leela_gpu.h): contexts, weight upload and
// layout, forward orchestration, CUDA-graph cache, batching server.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "lg_kernels.h"

// ------------------------------------------------------------------ errors

static thread_local std::string t_last_error;

void lg_set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    t_last_error = buf;
}

extern "C" const char *lg_last_error(void) { return t_last_error.c_str(); }

namespace {

using namespace lg;

constexpr int kMaxConv = 40;

// ------------------------------------------------------------ shapes

struct Shape {
    int k, cin, cout;
};

bool valid_desc(const lg_net_desc *d) {
    return d && d->c_in > 0 && d->c_in <= 64 && d->width1 > 0 && d->width > 0 && d->n3x3 >= 0 &&
           d->n3x3 < kMaxConv - 2 && (d->head_k == 1 || d->head_k == 3) &&
           (d->act == LG_ACT_ELU || d->act == LG_ACT_RELU) &&
           (!d->value_head || (d->fc_hidden > 0 && d->fc_hidden <= 4096)) && d->value_map >= 0 && d->value_map <= 2 &&
           d->precision >= LG_FP32 && d->precision <= LG_FP16;
}

std::vector<Shape> conv_shapes(const lg_net_desc *d) {
    std::vector<Shape> s;
    s.push_back({5, d->c_in, d->width1});
    for (int i = 0; i < d->n3x3; ++i) s.push_back({3, i == 0 ? d->width1 : d->width, d->width});
    s.push_back({d->head_k, d->n3x3 > 0 ? d->width : d->width1, 1});
    return s;
}

size_t weight_count(const lg_net_desc *d) {
    size_t n = 0;
    for (auto &s : conv_shapes(d)) n += (size_t)s.cout * s.cin * s.k * s.k + s.cout;
    if (d->value_head) n += (size_t)d->fc_hidden * kPoints + 2 * (size_t)d->fc_hidden + 1;
    return n;
}

// ------------------------------------------------------------ device memory

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

// ------------------------------------------------------------ nets

struct TcConv {
    __nv_bfloat16 *w = nullptr;  // [taps][halves][N][64]
    float *bias = nullptr;
    float *scale = nullptr;      // FP8 weights: per-output-channel scale
    int k, cin, cout, halves, ntaps;
};

struct Net {
    lg_net_desc d{};
    bool present = false;
    std::vector<Shape> shapes;
    // FP32 path
    std::vector<float *> wt;     // per trunk conv: [k*k][cin][cout]
    std::vector<float *> bias;
    float *head_w = nullptr;     // [k*k][cin]
    float head_b = 0.0f;
    float *w1s = nullptr, *b1 = nullptr, *w2 = nullptr;
    float b2 = 0.0f;
    // small-batch path (latency.cu): per conv layer and the head, weights
    // [8][cg][k*k][cout] with each split padded to `slice` floats
    bool lat_ok = false;
    std::vector<LatConv> lat;
    // tensor-core path
    std::vector<TcConv> tc;
    float *tc_head_w = nullptr;  // [width]
    // all 3x3 layers' weights back to back, for the persistent trunk kernel
    __nv_bfloat16 *trunk_w = nullptr;  // [n3x3][9][2][128][64]
    float *trunk_bias = nullptr, *trunk_scale = nullptr;
};

}  // namespace

struct lg_ctx {
    int device = 0;
    int max_batch = 0;
    int sm_count = 152;
    Net nets[2];
    cudaStream_t stream = nullptr;
    std::vector<void *> allocs;
    // FP32 buffers
    float *act[2] = {nullptr, nullptr};
    float *partial = nullptr;
    // small-batch path: partial sums, counters (zero between launches),
    // value-head partials
    float *lat_part = nullptr;
    int *lat_cnt = nullptr;
    float *lat_fcv = nullptr;
    // tensor-core buffers
    __nv_bfloat16 *l3[2] = {nullptr, nullptr};
    // the first layer's expanded input rows; a chunked device call alternates
    // l5 and l5b, so the next chunk is packed while a trunk reads the other
    __nv_bfloat16 *l5 = nullptr, *l5b = nullptr;
    int *d_err = nullptr;
    // shared
    uint8_t *d_planes = nullptr;
    // board-input calls: squares [B][361], to_move [B], then (4-aligned) moves [B][4] int32
    int8_t *d_boards = nullptr;
    float *d_logits = nullptr, *d_probs = nullptr, *d_value = nullptr;
    float *d_parts = nullptr;  // fused-head partial sums, [4][max_batch * 361]
    float *d_fcpart = nullptr; // value-head FC partial sums
    int *d_fccnt = nullptr;    // value-head group counters, zero between launches
    int *d_flags = nullptr;    // chunk flags and item counter of the persistent trunk kernel
    // pinned staging of the blocking calls, two slots so that chunk k+1 is
    // packed while chunk k runs: planes, outputs, logits, completion events
    uint8_t *h_planes = nullptr, *h_planes_b = nullptr;
    float *h_out = nullptr, *h_out2 = nullptr, *h_out_b = nullptr, *h_out2_b = nullptr;
    cudaEvent_t host_done[2] = {nullptr, nullptr};
    // board calls over several chunks of a tensor-core net (allocated on the
    // first such call): a ring of kPipe slots, each holding one super-chunk's
    // boards (pinned, device), input planes (device) and results (device,
    // pinned, with the error word); a stream for the copies
    static constexpr int kPipe = 4;
    cudaStream_t copy_stream = nullptr;
    size_t pl_in_bytes = 0, pl_out_floats = 0;
    uint8_t *pl_h_in = nullptr;
    int8_t *pl_d_in = nullptr;
    float *pl_d_out = nullptr, *pl_h_out = nullptr;
    uint8_t *pl_d_planes = nullptr;
    size_t pl_planes_bytes = 0;
    cudaEvent_t pl_h2d[kPipe] = {}, pl_comp[kPipe] = {}, pl_d2h[kPipe] = {};
    int planes_c = 0;
    std::mutex mu;
    std::map<std::tuple<int, int, uint32_t, int>, std::pair<cudaGraphExec_t, int>> graphs;
    // Per-kernel timing (device-pointer calls only): CUDA events around each
    // launch on the launching stream, resolved by lg_profile_read.
    bool profiling = false;
    std::vector<std::tuple<int, cudaEvent_t, cudaEvent_t>> prof_pending;
    std::vector<cudaEvent_t> event_pool;
    long long prof_launches[LG_PROF_KINDS] = {};
    double prof_ms[LG_PROF_KINDS] = {};
    // Kernel choice per power-of-two batch bucket (index = log2): [bucket][0]
    // 3x3 layers (and fused head) of the 128-wide tensor-core nets -- 0 =
    // 256-row transposed kernel, 1 = 128-row, 2 / 3 = persistent trunk --
    // or 4 = the whole net in the small-batch kernel (buckets up to
    // kLatMaxB, nets it supports; the default there); [bucket][1] first
    // layer, 0 = 256-row, 1 = 128-row.
    int tc_variant[17][2] = {};
    bool tuned = false;
    std::atomic<long long> launches{0};
    std::atomic<long long> batches{0};
    std::atomic<int> fault_in{0};
    // test hook (lg_inject_stall): the next launch of kernel kind stall_kind
    // (0 persistent trunk, 1 small-batch kernel) has one wait that nothing
    // satisfies, with its wait limits cut to stall_polls; -1 = disarmed
    int stall_kind = -1;
    uint32_t stall_polls = 0;
    // batching server
    struct Req {
        int net;
        const uint8_t *planes;
        int B;
        float temperature;
        float *out;
        void *tag;
    };
    // the worker's two pinned slots (separate from the blocking calls' buffers)
    uint8_t *srv_planes[2] = {nullptr, nullptr};
    float *srv_out[2] = {nullptr, nullptr};
    cudaEvent_t srv_done[2] = {nullptr, nullptr};
    std::thread worker;
    std::mutex qmu;
    std::condition_variable qcv, dcv;
    std::deque<Req> queue;
    std::deque<void *> done;
    bool stop = false;
    bool worker_started = false;
    int worker_error = 0;
};

namespace {

template <class T>
int dev_alloc(lg_ctx *c, T **p, size_t count) {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) {
        lg_set_error("cudaMalloc(%zu bytes): %s", count * sizeof(T), cudaGetErrorString(e));
        *p = nullptr;
        return LG_ERR_ALLOC;
    }
    c->allocs.push_back(*p);
    return LG_OK;
}

template <class T>
int upload(lg_ctx *c, T **p, const std::vector<T> &h) {
    int rc = dev_alloc(c, p, h.size());
    if (rc) return rc;
    LG_CUDA_TRY(cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return LG_OK;
}

bool tc_supported(const lg_net_desc *d) {
    return d->c_in <= 32 && d->width1 == d->width && (d->width == 64 || d->width == 128) &&
           d->head_k == 1 && d->n3x3 >= 1;
}

// A weight rounded to nearest even in the tensor-core operand type (FP16 for
// LG_FP16 nets, else BF16), as its 16 bits in a BF16-typed slot.
__nv_bfloat16 operand16(float v, bool f16) {
    if (!f16) return __float2bfloat16(v);
    const __half h = __float2half_rn(v);
    __nv_bfloat16 b;
    std::memcpy(&b, &h, sizeof b);
    return b;
}

// The value of that rounding, back in FP32 (weights the FP32 heads use).
float round_operand(float v, bool f16) {
    return f16 ? __half2float(__float2half_rn(v)) : __bfloat162float(__float2bfloat16(v));
}

// E4M3 round-to-nearest-even with saturation at 448 (the quantiser of the
// FP8-weight variant; E4M3 values are exact in BF16).
float e4m3_round(float x) {
    if (x != x) return x;
    float a = std::fabs(x);
    if (a >= 448.0f) return x < 0 ? -448.0f : 448.0f;
    if (a == 0.0f) return x;
    int e;
    std::frexp(a, &e);
    int ex = std::max(e - 1, -6);
    float step = std::ldexp(1.0f, ex - 3);
    float q = std::nearbyint(a / step) * step;
    q = std::min(q, 448.0f);
    return x < 0 ? -q : q;
}

// The small-batch kernel's weight layout, for the shapes it covers: every
// layer's input channels split 8 ways (cin % 8 == 0, and after the first
// layer 4-channel groups: cin % 32 == 0), at most 128 output channels (even,
// or the head's one), 1x1 / 3x3 / 5x5 filters, the staged input and the
// weight slice within the kernel's shared memory, and for value nets an FC
// layer of at most 256 units in 8 equal slices.  Other nets keep the
// generic path at every batch size.
int build_lat(lg_ctx *c, Net &n, const std::vector<std::vector<float>> &Wraw) {
    const lg_net_desc &d = n.d;
    const int nl = (int)n.shapes.size();
    bool ok = nl <= kLatMaxLayers && (!d.value_head || (d.fc_hidden % kLatSplits == 0 && d.fc_hidden <= 256));
    for (int l = 0; l < nl && ok; ++l) {
        const Shape sh = n.shapes[l];
        const int cg = sh.cin / kLatSplits;
        const int slice = (cg * sh.k * sh.k * sh.cout + 3) & ~3;
        ok = sh.cin % kLatSplits == 0 && (l == 0 || cg % 4 == 0) && cg <= kLatMaxCg && cg * sh.k <= kLatMaxCg * 5 &&
             (sh.k == 1 || sh.k == 3 || sh.k == 5) && sh.cout <= 128 && (sh.cout % 2 == 0 || sh.cout == 1) &&
             slice <= kLatSliceMax;
    }
    if (!ok) return LG_OK;
    for (int l = 0; l < nl; ++l) {
        const Shape sh = n.shapes[l];
        const int kk = sh.k * sh.k, cg = sh.cin / kLatSplits;
        LatConv L{};
        L.k = sh.k;
        L.cin = sh.cin;
        L.cout = sh.cout;
        L.cg = cg;
        L.slice = (cg * kk * sh.cout + 3) & ~3;
        std::vector<float> w((size_t)kLatSplits * L.slice, 0.0f);
        for (int sp = 0; sp < kLatSplits; ++sp)
            for (int cl = 0; cl < cg; ++cl)
                for (int t = 0; t < kk; ++t)
                    for (int o = 0; o < sh.cout; ++o)
                        w[(size_t)sp * L.slice + ((size_t)cl * kk + t) * sh.cout + o] =
                            Wraw[l][((size_t)o * sh.cin + sp * cg + cl) * kk + t];
        float *dw;
        int rc = upload(c, &dw, w);
        if (rc) return rc;
        L.w = dw;
        L.bias = l + 1 < nl ? n.bias[l] : nullptr;
        n.lat.push_back(L);
    }
    n.lat_ok = true;
    return LG_OK;
}

// The small-batch kernel's layout for tensor-core nets of width 128 (1x1
// head): the first layer and the head in FP32 on the weights as the
// precision rounds them (FP8: the E4M3 codes, the per-channel scale being
// applied by the consumer), the 3x3 layers as 16-bit [8][9][128][16] for the
// warp MMA.  Biases and scales are the tensor-core path's own arrays.
int build_lat_tc(lg_ctx *c, Net &n, const std::vector<std::vector<float>> &Wraw) {
    const lg_net_desc &d = n.d;
    const int nl = (int)n.shapes.size();
    const bool fp8 = d.precision == LG_FP8W, f16 = d.precision == LG_FP16;
    if (d.width != 128 || d.width1 != 128 || d.c_in % kLatSplits != 0 || d.head_k != 1 || nl > kLatMaxLayers ||
        (d.value_head && (d.fc_hidden % kLatSplits != 0 || d.fc_hidden > 256)) || d.c_in / kLatSplits * 5 > kLatMaxCg * 5)
        return LG_OK;
    for (int l = 0; l < nl; ++l) {
        const Shape sh = n.shapes[l];
        const int kk = sh.k * sh.k, cg = sh.cin / kLatSplits;
        const bool head = l + 1 == nl, mid = l > 0 && !head;
        std::vector<float> scale(sh.cout, 1.0f);
        if (fp8 && !head)
            for (int o = 0; o < sh.cout; ++o) {
                float m = 0.0f;
                for (size_t i = 0; i < (size_t)sh.cin * kk; ++i) m = std::max(m, std::fabs(Wraw[l][(size_t)o * sh.cin * kk + i]));
                scale[o] = m > 0.0f ? m / 448.0f : 1.0f;
            }
        // the weight as the path computes with it
        auto wv = [&](int o, int ci, int t) {
            const float v = Wraw[l][((size_t)o * sh.cin + ci) * kk + t];
            if (head) return round_operand(v, f16);
            return fp8 ? e4m3_round(v / scale[o]) : round_operand(v, f16);
        };
        LatConv L{};
        L.k = sh.k;
        L.cin = sh.cin;
        L.cout = sh.cout;
        L.cg = cg;
        L.mma = mid ? 1 : 0;
        L.bias = head ? nullptr : n.tc[l].bias;
        L.scale = head ? nullptr : n.tc[l].scale;
        int rc;
        if (mid) {
            L.slice = 9 * 128 * 16 / 2;
            std::vector<__nv_bfloat16> w((size_t)kLatSplits * 9 * 128 * 16);
            for (int sp = 0; sp < kLatSplits; ++sp)
                for (int t = 0; t < 9; ++t)
                    for (int o = 0; o < 128; ++o)
                        for (int cl = 0; cl < 16; ++cl)
                            w[(((size_t)sp * 9 + t) * 128 + o) * 16 + cl] = operand16(wv(o, sp * 16 + cl, t), f16);
            __nv_bfloat16 *dw;
            if ((rc = upload(c, &dw, w))) return rc;
            L.w = dw;
        } else {
            L.slice = (cg * kk * sh.cout + 3) & ~3;
            std::vector<float> w((size_t)kLatSplits * L.slice, 0.0f);
            for (int sp = 0; sp < kLatSplits; ++sp)
                for (int cl = 0; cl < cg; ++cl)
                    for (int t = 0; t < kk; ++t)
                        for (int o = 0; o < sh.cout; ++o)
                            w[(size_t)sp * L.slice + ((size_t)cl * kk + t) * sh.cout + o] = wv(o, sp * cg + cl, t);
            float *dw;
            if ((rc = upload(c, &dw, w))) return rc;
            L.w = dw;
        }
        n.lat.push_back(L);
    }
    n.lat_ok = true;
    return LG_OK;
}

int build_net(lg_ctx *c, Net &n, const lg_net_desc *d) {
    if (!valid_desc(d) || !d->weights) {
        lg_set_error("invalid network description");
        return LG_ERR_ARG;
    }
    if (d->precision != LG_FP32 && !tc_supported(d)) {
        lg_set_error("BF16/FP16/FP8 paths need c_in <= 32, width1 == width in {64,128}, head_k == 1");
        return LG_ERR_ARG;
    }
    n.d = *d;
    n.d.weights = nullptr;
    n.present = true;
    n.shapes = conv_shapes(d);
    const float *w = d->weights;
    size_t off = 0;
    int ntrunk = (int)n.shapes.size() - 1;
    std::vector<std::vector<float>> Wraw(n.shapes.size()), Braw(n.shapes.size());
    for (size_t l = 0; l < n.shapes.size(); ++l) {
        auto s = n.shapes[l];
        size_t nw = (size_t)s.cout * s.cin * s.k * s.k;
        Wraw[l].assign(w + off, w + off + nw);
        Braw[l].assign(w + off + nw, w + off + nw + s.cout);
        off += nw + s.cout;
    }
    int rc;
    // ---- FP32 layouts: W[o][c][ky][kx] -> wt[tap][c][o]
    if (d->precision == LG_FP32) {
        for (int l = 0; l < ntrunk; ++l) {
            auto s = n.shapes[l];
            int kk = s.k * s.k;
            std::vector<float> wt((size_t)kk * s.cin * s.cout);
            for (int o = 0; o < s.cout; ++o)
                for (int ci = 0; ci < s.cin; ++ci)
                    for (int t = 0; t < kk; ++t)
                        wt[((size_t)t * s.cin + ci) * s.cout + o] =
                            Wraw[l][((size_t)o * s.cin + ci) * kk + t];
            float *dw, *db;
            if ((rc = upload(c, &dw, wt)) || (rc = upload(c, &db, Braw[l]))) return rc;
            n.wt.push_back(dw);
            n.bias.push_back(db);
        }
        auto hs = n.shapes.back();
        int kk = hs.k * hs.k;
        std::vector<float> wh((size_t)kk * hs.cin);
        for (int ci = 0; ci < hs.cin; ++ci)
            for (int t = 0; t < kk; ++t) wh[(size_t)t * hs.cin + ci] = Wraw.back()[(size_t)ci * kk + t];
        if ((rc = upload(c, &n.head_w, wh))) return rc;
        n.head_b = Braw.back()[0];
        if ((rc = build_lat(c, n, Wraw))) return rc;
    } else {
        // ---- tensor-core layouts: [tap][half][N][64] 16-bit operands (BF16,
        // or FP16 for LG_FP16), K-major rows.
        bool fp8 = d->precision == LG_FP8W;
        const bool f16 = d->precision == LG_FP16;
        for (int l = 0; l < ntrunk; ++l) {
            auto s = n.shapes[l];
            TcConv t{};
            t.k = s.k;
            t.cin = s.cin;
            t.cout = s.cout;
            t.ntaps = (l == 0) ? 5 : 9;
            // First layer: K of each vertical tap dy = the 5 horizontal taps
            // dx x c_in channels (channel index dx*c_in + c), padded to 64s.
            int kper = (l == 0) ? 5 * s.cin : s.cin;
            t.halves = (kper + 63) / 64;
            std::vector<float> scale(s.cout, 1.0f);
            int kk = s.k * s.k;
            if (fp8) {
                for (int o = 0; o < s.cout; ++o) {
                    float m = 0.0f;
                    for (size_t i = 0; i < (size_t)s.cin * kk; ++i)
                        m = std::max(m, std::fabs(Wraw[l][(size_t)o * s.cin * kk + i]));
                    scale[o] = m > 0.0f ? m / 448.0f : 1.0f;
                }
            }
            std::vector<__nv_bfloat16> wb((size_t)t.ntaps * t.halves * s.cout * 64,
                                          __float2bfloat16(0.0f));
            for (int tap = 0; tap < t.ntaps; ++tap)
                for (int o = 0; o < s.cout; ++o)
                    for (int kidx = 0; kidx < t.halves * 64; ++kidx) {
                        float v = 0.0f;
                        if (l == 0) {
                            int dx = kidx / s.cin, ci = kidx % s.cin;
                            if (kidx < 5 * s.cin)
                                v = Wraw[l][((size_t)o * s.cin + ci) * kk + tap * 5 + dx];
                        } else if (kidx < s.cin) {
                            v = Wraw[l][((size_t)o * s.cin + kidx) * kk + tap];
                        }
                        if (fp8) v = e4m3_round(v / scale[o]);
                        int half = kidx / 64;
                        wb[(((size_t)tap * t.halves + half) * s.cout + o) * 64 + kidx % 64] =
                            operand16(v, f16);
                    }
            if ((rc = upload(c, &t.w, wb)) || (rc = upload(c, &t.bias, Braw[l]))) return rc;
            if (fp8 && (rc = upload(c, &t.scale, scale))) return rc;
            n.tc.push_back(t);
        }
        // The 3x3 layers again as one array for the persistent trunk kernel.
        if (d->width == 128 && ntrunk > 1) {
            const size_t per = (size_t)9 * 2 * 128 * 64;
            const int nl = ntrunk - 1;
            rc = dev_alloc(c, &n.trunk_w, per * nl);
            if (!rc) rc = dev_alloc(c, &n.trunk_bias, (size_t)nl * 128);
            if (!rc && fp8) rc = dev_alloc(c, &n.trunk_scale, (size_t)nl * 128);
            if (rc) return rc;
            for (int l = 1; l < ntrunk; ++l) {
                const TcConv &t = n.tc[l];
                LG_CUDA_TRY(cudaMemcpy(n.trunk_w + per * (l - 1), t.w, per * sizeof(__nv_bfloat16),
                                       cudaMemcpyDeviceToDevice));
                LG_CUDA_TRY(cudaMemcpy(n.trunk_bias + 128 * (l - 1), t.bias, 128 * sizeof(float),
                                       cudaMemcpyDeviceToDevice));
                if (fp8)
                    LG_CUDA_TRY(cudaMemcpy(n.trunk_scale + 128 * (l - 1), t.scale, 128 * sizeof(float),
                                           cudaMemcpyDeviceToDevice));
            }
        }
        // Fused 1x1 head weights, rounded to the operand type as the
        // precision states.
        std::vector<float> hw(Wraw.back());
        for (auto &v : hw) v = round_operand(v, f16);
        if ((rc = upload(c, &n.tc_head_w, hw))) return rc;
        n.head_b = Braw.back()[0];
        if ((rc = build_lat_tc(c, n, Wraw))) return rc;
    }
    if (d->value_head) {
        int H = d->fc_hidden;
        const float *W1 = w + off;
        // W1 [H][361] stored sliced by hidden units: [H/U][361][U], U = 64,
        // zero-padded past H, so one FC1 tile's weights are one block.
        const int U = value_fc_slice_units(), slices = (H + U - 1) / U;
        std::vector<float> w1s((size_t)slices * kPoints * U, 0.0f), b1(W1 + (size_t)H * kPoints,
                                                                      W1 + (size_t)H * kPoints + H);
        std::vector<float> w2(W1 + (size_t)H * kPoints + H, W1 + (size_t)H * kPoints + 2 * H);
        const bool lowp = d->precision != LG_FP32, f16 = d->precision == LG_FP16;
        for (int o = 0; o < H; ++o)
            for (int i = 0; i < kPoints; ++i) {
                float v = W1[(size_t)o * kPoints + i];
                if (lowp) v = round_operand(v, f16);
                w1s[((size_t)(o / U) * kPoints + i) * U + o % U] = v;
            }
        if (lowp)
            for (auto &v : w2) v = round_operand(v, f16);
        n.b2 = W1[(size_t)H * kPoints + 2 * H];
        if ((rc = upload(c, &n.w1s, w1s)) || (rc = upload(c, &n.b1, b1)) ||
            (rc = upload(c, &n.w2, w2)))
            return rc;
    }
    return LG_OK;
}

int check_fault(lg_ctx *c) {
    int f = c->fault_in.load();
    if (f > 0) {
        if (c->fault_in.fetch_sub(1) == 1) {
            lg_set_error("injected fault");
            return LG_ERR_CUDA;
        }
    }
    return LG_OK;
}

// ------------------------------------------------------------ forward

cudaEvent_t pool_event(lg_ctx *c) {
    if (!c->event_pool.empty()) {
        cudaEvent_t e = c->event_pool.back();
        c->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Brackets one kernel launch with events when profiling is on.
struct ProfScope {
    lg_ctx *c;
    int kind;
    cudaStream_t s;
    cudaEvent_t a = nullptr, b = nullptr;
    ProfScope(lg_ctx *c_, bool on, int kind_, cudaStream_t s_) : c(on ? c_ : nullptr), kind(kind_), s(s_) {
        if (c) {
            a = pool_event(c);
            b = pool_event(c);
            cudaEventRecord(a, s);
        }
    }
    ~ProfScope() {
        if (c) {
            cudaEventRecord(b, s);
            c->prof_pending.emplace_back(kind, a, b);
        }
    }
};

// Bucket index of batch B (log2 of the next power of two).
int bucket_of(int B) {
    int bl = 0;
    while ((1 << bl) < B && bl < 16) ++bl;
    return bl;
}

bool use_lat(lg_ctx *c, const Net &n, int B) {
    return n.lat_ok && B <= kLatMaxB && c->lat_part && c->tc_variant[bucket_of(B)][0] == 4;
}

// Kernel choices without tuning (measured on GB300, policy + value pairs,
// device-resident inputs): FP32 nets run the small-batch kernel up to 8
// positions (B = 8: 1.12 against 1.13 ms on the per-layer kernels); 16-bit
// nets run it up to 2 (B = 2: 220 against 254 us on the persistent trunk;
// B = 3: 314 against 256 us) and the persistent trunk with the first layer
// inside from 3 positions on (B = 256: 0.43 against 0.76 ms a pair on the
// per-layer kernels).  A context with a 16-bit net takes the 16-bit rule.
void default_tuning(lg_ctx *c) {
    bool lowp = false;
    for (const Net &n : c->nets) lowp = lowp || (n.present && n.d.precision != LG_FP32);
    for (int b = 0; b < 17; ++b) {
        c->tc_variant[b][0] = lowp ? ((1 << b) <= 2 ? 4 : 3) : ((1 << b) <= kLatMaxB ? 4 : 0);
        c->tc_variant[b][1] = 0;
    }
}

int forward_lat(lg_ctx *c, Net &n, const uint8_t *planes, int B, float T, float *probs, float *logits_out,
                float *value, cudaStream_t s, int *nlaunch, bool prof) {
    const lg_net_desc &d = n.d;
    LatParams p{};
    p.nl = (int)n.lat.size();
    for (int l = 0; l < p.nl; ++l) p.L[l] = n.lat[l];
    p.B = B;
    p.c_in = d.c_in;
    p.act = d.act;
    p.act_head = d.act_head;
    p.head_b = n.head_b;
    p.planes = planes;
    p.part = c->lat_part;
    p.cnt = c->lat_cnt;
    p.err = c->d_err;
    p.temperature = T;
    p.probs = probs;
    p.logits_out = logits_out;
    p.value_head = d.value_head;
    p.w1s = n.w1s;
    p.b1 = n.b1;
    p.w2 = n.w2;
    p.b2 = n.b2;
    p.H = d.fc_hidden;
    p.value_map = d.value_map;
    p.value = value;
    p.fcv = c->lat_fcv;
    p.stall_row = -1;
    if (c->stall_kind == 1) {
        p.stall_row = 0;
        p.poll_limit = c->stall_polls;
        c->stall_kind = -1;
    }
    int rc;
    {
        ProfScope ps(c, prof, LG_PROF_LAT, s);
        const int mode = d.precision == LG_FP32 ? 0 : (d.precision == LG_FP16 ? 2 : 1);
        rc = launch_lat(p, mode, c->sm_count, s);
    }
    *nlaunch = 1;
    return rc;
}

int forward_fp32(lg_ctx *c, Net &n, const uint8_t *planes, int B, float T, float *probs,
                 float *logits_out, float *value, cudaStream_t s, int *nlaunch, bool prof) {
    if (use_lat(c, n, B)) return forward_lat(c, n, planes, B, T, probs, logits_out, value, s, nlaunch, prof);
    const lg_net_desc &d = n.d;
    int L = 0;
    {
        ProfScope ps(c, prof, LG_PROF_OTHER, s);
        launch_pack_planes_f32(planes, B, d.c_in, c->act[0], s);
    }
    ++L;
    int cur = 0;
    int ntrunk = (int)n.shapes.size() - 1;
    for (int l = 0; l < ntrunk; ++l) {
        auto sh = n.shapes[l];
        ProfScope ps(c, prof, LG_PROF_FP32_CONV, s);
        launch_conv_f32(c->act[cur], n.wt[l], n.bias[l], c->act[cur ^ 1], B, sh.cin, sh.cout, sh.k,
                        d.act, c->partial, s);
        L += conv_f32_partial_floats(B, sh.cin, sh.cout, sh.k) ? 2 : 1;
        cur ^= 1;
    }
    auto hs = n.shapes.back();
    float *lg = logits_out ? logits_out : c->d_logits;
    {
        ProfScope ps(c, prof, LG_PROF_OTHER, s);
        launch_head_conv_f32(c->act[cur], n.head_w, n.head_b, B, hs.cin, hs.k, d.act_head, d.act, lg, s);
    }
    ++L;
    {
        ProfScope ps(c, prof, LG_PROF_TAIL, s);
        HeadIn h{lg, 1, 0, 0.0f, 0, d.act, nullptr};
        if (!d.value_head)
            launch_softmax(h, B, T, probs, s);
        else
            launch_value_fc(h, B, n.w1s, n.b1, n.w2, n.b2, d.fc_hidden, d.act, d.value_map, value,
                            c->d_fcpart, c->d_fccnt, s);
    }
    ++L;
    *nlaunch = L;
    return LG_OK;
}

// l5_ready: the first layer's expanded input rows are already in c->l5 (the
// board path's gather writes them), so `planes` is not read.
// count (device, optional): only the first *count - count_base of the B
// positions are computed -- a batch whose size is known only on the device
// (the gated path); it runs on the persistent trunk with the first layer
// inside it, which a net must support (trunk_fusable).
bool trunk_fusable(const Net &n) {
    return n.trunk_w != nullptr && n.tc.size() >= 2 && n.tc[0].k == 5 && n.tc[0].halves == 2 &&
           n.tc[0].cout == 128;
}

// next (optional): the following batch's planes, packed by CTAs of this
// batch's finish launch into next->out, which must not be this batch's l5.
// mid (optional): launches made between the layers and the finish (the
// board pipeline's gather of the next chunk).
// l5buf: this batch's first-layer rows (default c->l5).  pdl: the trunk and
// the finish are launched as programmatic dependents of the kernel before
// them (the trunk's prologue overlaps that kernel's end, the packing CTAs
// of the finish start as the trunk's CTAs leave).
int forward_tc(lg_ctx *c, Net &n, const uint8_t *planes, int B, float T, float *probs,
               float *logits_out, float *value, cudaStream_t s, int *nlaunch, bool prof,
               bool l5_ready = false, const int *count = nullptr, int count_base = 0,
               const PackJob *next = nullptr, __nv_bfloat16 *l5buf = nullptr, bool pdl = false,
               const std::function<int()> *mid = nullptr) {
    __nv_bfloat16 *const L5 = l5buf ? l5buf : c->l5;
    if (!count && use_lat(c, n, B) && !l5_ready)
        return forward_lat(c, n, planes, B, T, probs, logits_out, value, s, nlaunch, prof);
    if (count && !trunk_fusable(n)) {
        lg_set_error("a device-side batch size needs a 128-wide tensor-core net with a 5x5 first layer");
        return LG_ERR_ARG;
    }
    const lg_net_desc &d = n.d;
    const int f16 = d.precision == LG_FP16 ? 1 : 0;
    int L = 0;
    const TcConv &first = n.tc[0];
    if (!l5_ready) {
        ProfScope ps(c, prof, LG_PROF_PACK, s);
        launch_pack_planes_l5(planes, B, d.c_in, first.halves, f16 != 0, L5, s, count, count_base);
        ++L;
    }
    float *lg = logits_out ? logits_out : c->d_logits;
    const size_t part_stride = (size_t)B * kPoints;
    int bl = 0;
    while ((1 << bl) < B && bl < 16) ++bl;
    const int var3 = count ? 3 : c->tc_variant[bl][0], var1 = c->tc_variant[bl][1];
    const bool use_trunk = (var3 == 2 || var3 == 3) && n.trunk_w != nullptr;
    // choice 3: the 5x5 first layer runs inside the trunk launch too
    const bool fuse_first = use_trunk && var3 == 3 && trunk_fusable(n);
    int cur = 0;
    for (size_t l = fuse_first ? 1 : 0; l < n.tc.size(); ++l) {
        const TcConv &t = n.tc[l];
        const bool last = l + 1 == n.tc.size();
        if (use_trunk && l == 1) {
            // layers 1 .. end in one persistent launch; layer 0 wrote l3[0]
            // (or runs as the launch's first items)
            TcTrunk tt{};
            if (fuse_first) {
                tt.buf5 = L5;
                tt.rows5 = B * kL5Board;
                tt.w0 = first.w;
                tt.bias0 = first.bias;
                tt.scale0 = first.scale;
            }
            tt.buf_a = c->l3[0];
            tt.buf_b = c->l3[1];
            tt.w = n.trunk_w;
            tt.bias = n.trunk_bias;
            tt.scale = n.trunk_scale;
            tt.head_w = n.tc_head_w;
            tt.act = d.act;
            tt.rows = B * kL3Board;
            tt.nl = (int)n.tc.size() - 1;
            tt.f16 = f16;
            tt.count = count;
            tt.count_base = count_base;
            tt.pdl = pdl;
            if (c->stall_kind == 0) {
                // the first item of the second 3x3 layer
                tt.stall_item = trunk_layer_item(tt.rows, fuse_first ? tt.rows5 : 0, 1);
                tt.wait_limit = tt.poll_limit = c->stall_polls;
                c->stall_kind = -1;
            }
            int rc;
            {
                ProfScope ps(c, prof, LG_PROF_TC_TRUNK, s);
                rc = launch_tc_trunk(tt, c->d_parts, part_stride, c->d_flags, c->d_err, s, c->sm_count);
            }
            if (rc) return rc;
            L += 1;
            break;
        }
        TcLayer tl{};
        tl.in = (l == 0) ? (const void *)L5 : (const void *)c->l3[cur];
        tl.w = t.w;
        tl.bias = t.bias;
        tl.scale = t.scale;
        tl.head_w = last ? n.tc_head_w : nullptr;
        tl.act = d.act;
        tl.cin_halves = t.halves;
        tl.n = t.cout;
        tl.in_kind = (l == 0) ? 1 : 0;
        tl.rows = (l == 0) ? B * kL5Board : B * kL3Board;
        tl.variant = (l == 0) ? var1 : var3;
        tl.f16 = f16;
        __nv_bfloat16 *out = (l == 0) ? c->l3[0] : c->l3[cur ^ 1];
        int rc;
        {
            ProfScope ps(c, prof, l == 0 ? LG_PROF_TC_FIRST : (last ? LG_PROF_TC_HEAD : LG_PROF_TC_3X3), s);
            rc = launch_tc_conv(tl, last ? nullptr : out, last ? c->d_parts : nullptr, part_stride,
                                c->d_err, s, c->sm_count);
        }
        if (rc) return rc;
        ++L;
        if (l > 0) cur ^= 1;
    }
    if (mid) {
        const int rc = (*mid)();
        if (rc) return rc;
    }
    {
        ProfScope ps(c, prof, LG_PROF_TAIL, s);
        HeadIn h{c->d_parts, tc_head_parts(d.width, use_trunk ? 0 : var3), part_stride, n.head_b, d.act_head,
                 d.act, lg, count, count_base};
        if (next) {
            FinishJob j{};
            j.h = h;
            j.B = B;
            j.value_head = d.value_head;
            j.temperature = T;
            j.probs = probs;
            j.w1s = n.w1s;
            j.b1 = n.b1;
            j.w2 = n.w2;
            j.b2 = n.b2;
            j.H = d.fc_hidden;
            j.act = d.act;
            j.value_map = d.value_map;
            j.value = value;
            j.part = c->d_fcpart;
            j.cnt = c->d_fccnt;
            launch_finish_pack(j, *next, s, pdl);
        } else if (!d.value_head) {
            launch_softmax(h, B, T, probs, s, nullptr, pdl);
        } else {
            launch_value_fc(h, B, n.w1s, n.b1, n.w2, n.b2, d.fc_hidden, d.act, d.value_map, value,
                            c->d_fcpart, c->d_fccnt, s, pdl);
        }
    }
    L += (next && d.value_head) ? 2 : 1;  // a value head with the next chunk's packing: two launches
    *nlaunch = L;
    return LG_OK;
}

int forward(lg_ctx *c, int net, const uint8_t *planes, int B, float T, float *probs,
            float *logits, float *value, cudaStream_t s, int *nlaunch, bool prof = false,
            bool l5_ready = false, const PackJob *next = nullptr, __nv_bfloat16 *l5buf = nullptr,
            bool pdl = false) {
    Net &n = c->nets[net];
    if (n.d.precision == LG_FP32)
        return forward_fp32(c, n, planes, B, T, probs, logits, value, s, nlaunch, prof);
    return forward_tc(c, n, planes, B, T, probs, logits, value, s, nlaunch, prof, l5_ready, nullptr, 0, next,
                      l5buf, pdl);
}

// ----------------------------------------------------- board-call pipeline

int run_device(lg_ctx *c, int net, const uint8_t *planes, int B, float T, float *probs, float *logits,
               float *value, cudaStream_t s);

constexpr int kPipeMaxBatch = 4096;    // larger contexts keep the per-chunk graphs
constexpr int kPipeSuperTarget = 2048; // positions per super-chunk (a multiple of max_batch)

size_t pipe_mv_off(size_t n) { return (n * (kPoints + 1) + 3) & ~(size_t)3; }

int pipe_super(const lg_ctx *c) { return c->max_batch * std::max(1, kPipeSuperTarget / c->max_batch); }

int pipe_alloc(lg_ctx *c) {
    if (c->pl_d_in) return LG_OK;
    constexpr int R = lg_ctx::kPipe;
    const size_t S = (size_t)pipe_super(c);
    c->pl_in_bytes = (pipe_mv_off(S) + S * 16 + 255) & ~(size_t)255;
    c->pl_out_floats = (2 * S * kPoints + 64 + 63) & ~(size_t)63;  // probs, logits, the error word
    c->pl_planes_bytes = (S * (size_t)c->planes_c * kPoints + 255) & ~(size_t)255;
    // each resource is made once, so a call after a failed one (out of
    // pinned memory, say) neither leaks nor repeats what was made
    if (!c->copy_stream && cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
        c->copy_stream = nullptr;
        lg_set_error("board pipeline: stream creation failed");
        return LG_ERR_CUDA;
    }
    for (int r = 0; r < R; ++r)
        for (cudaEvent_t *e : {&c->pl_h2d[r], &c->pl_comp[r], &c->pl_d2h[r]})
            if (!*e && cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) {
                *e = nullptr;
                lg_set_error("board pipeline: event creation failed");
                return LG_ERR_CUDA;
            }
    if ((!c->pl_h_in && cudaMallocHost(&c->pl_h_in, R * c->pl_in_bytes) != cudaSuccess) ||
        (!c->pl_h_out && cudaMallocHost(&c->pl_h_out, R * c->pl_out_floats * sizeof(float)) != cudaSuccess)) {
        lg_set_error("board pipeline: cudaMallocHost failed");
        return LG_ERR_ALLOC;
    }
    if (!c->pl_d_out)
        if (int rc = dev_alloc(c, &c->pl_d_out, R * c->pl_out_floats)) return rc;
    if (!c->pl_d_planes)
        if (int rc = dev_alloc(c, &c->pl_d_planes, R * c->pl_planes_bytes)) return rc;
    // pl_d_in last: its presence marks the pipeline as complete
    int8_t *din = nullptr;
    if (int rc = dev_alloc(c, &din, R * c->pl_in_bytes)) return rc;
    c->pl_d_in = din;
    return LG_OK;
}

// Board calls of a tensor-core net over more than one chunk, in super-chunks
// of pipe_super(c) positions (a multiple of max_batch) through a ring of
// kPipe slots.  For super-chunk j (slot j % kPipe): the host copies its
// boards into the slot's pinned buffer and the copy stream moves them to the
// device; the compute stream gathers the input planes of all its boards in
// one launch (one CTA a board: enough boards to fill the GPU, where a
// chunk's 256 would leave it waiting on one CTA's latency), then runs the
// chained device path over them (run_device: per chunk the trunk, then the
// head with the next chunk's packing, as programmatic dependents); the copy
// stream brings the results and the error word back, and the host hands
// them out one super-chunk later, while the GPU works on the next.
int run_host_boards_pipe(lg_ctx *c, int net, int B, float T, float *probs, float *logits, float *value,
                         const int8_t *squares, const int8_t *to_move, const int32_t *moves) {
    constexpr int R = lg_ctx::kPipe;
    Net &n = c->nets[net];
    if (int rc = pipe_alloc(c)) return rc;
    // Super-chunks of S positions, except the first and the last ones: the
    // GPU waits for the first one's boards and gather, so it is one chunk;
    // the host copies the last super-chunk's results out after the GPU is
    // done, so the call ends with one of at most an eighth of S, the rest of
    // the remainder before it.  Every super-chunk starts on a multiple of
    // max_batch, so the chunks are those of the plane-input calls (a ragged
    // last chunk included) and so are the results, bit for bit.
    const int S = pipe_super(c);
    std::vector<int> sb{0};  // super-chunk starts, then B
    {
        const int mb = c->max_batch;
        const int q = std::max(mb, S / 8 / mb * mb);
        int b = 0;
        if (S > mb && B - b > mb + S + q) sb.push_back(b += mb);
        while (B - b > S + q) sb.push_back(b += S);
        const int last = (B - q + mb - 1) / mb * mb;
        if (last > b && last < B) sb.push_back(b = last);
        sb.push_back(B);
    }
    const int nsup = (int)sb.size() - 1;
    const bool with_moves = n.d.c_in > 24, want_logits = logits != nullptr && !n.d.value_head;
    const int which = net == LG_NET_POLICY ? 0 : 1;
    const size_t mv_off = pipe_mv_off((size_t)S);
    cudaStream_t s = c->stream, cs = c->copy_stream;
    auto nb_of = [&](int j) { return sb[j + 1] - sb[j]; };
    auto din = [&](int j) { return c->pl_d_in + (size_t)(j % R) * c->pl_in_bytes; };
    auto hin = [&](int j) { return c->pl_h_in + (size_t)(j % R) * c->pl_in_bytes; };
    auto dpl = [&](int j) { return c->pl_d_planes + (size_t)(j % R) * c->pl_planes_bytes; };
    auto dout = [&](int j) { return c->pl_d_out + (size_t)(j % R) * c->pl_out_floats; };
    auto hout = [&](int j) { return c->pl_h_out + (size_t)(j % R) * c->pl_out_floats; };
    const size_t err_off = 2 * (size_t)S * kPoints;
    auto stage_in = [&](int j) -> int {
        const int nb = nb_of(j), b0 = sb[j];
        uint8_t *h = hin(j);
        std::memcpy(h, squares + (size_t)b0 * kPoints, (size_t)nb * kPoints);
        std::memcpy(h + (size_t)S * kPoints, to_move + b0, (size_t)nb);
        if (with_moves) std::memcpy(h + mv_off, moves + (size_t)b0 * 4, (size_t)nb * 16);
        LG_CUDA_TRY(cudaMemcpyAsync(din(j), h, c->pl_in_bytes, cudaMemcpyHostToDevice, cs));
        LG_CUDA_TRY(cudaEventRecord(c->pl_h2d[j % R], cs));
        return LG_OK;
    };
    auto launch = [&](int j) -> int {
        const int nb = nb_of(j);
        const int8_t *d = din(j), *dtm = d + (size_t)S * kPoints;
        const int32_t *dmv = with_moves ? reinterpret_cast<const int32_t *>(d + mv_off) : nullptr;
        LG_CUDA_TRY(cudaStreamWaitEvent(s, c->pl_h2d[j % R], 0));
        if (int rc = launch_gather(d, dtm, dmv, nb, which, n.d.c_in, dpl(j), s)) return rc;
        ++c->launches;
        float *o = dout(j);
        if (int rc = run_device(c, net, dpl(j), nb, T, o, want_logits ? o + (size_t)S * kPoints : nullptr, o, s))
            return rc;
        // the results (and the error word) back on the copy stream
        float *h = hout(j);
        const size_t nout = n.d.value_head ? (size_t)nb : (size_t)nb * kPoints;
        LG_CUDA_TRY(cudaEventRecord(c->pl_comp[j % R], s));
        LG_CUDA_TRY(cudaStreamWaitEvent(cs, c->pl_comp[j % R], 0));
        LG_CUDA_TRY(cudaMemcpyAsync(h, o, nout * sizeof(float), cudaMemcpyDeviceToHost, cs));
        if (want_logits)
            LG_CUDA_TRY(cudaMemcpyAsync(h + (size_t)S * kPoints, o + (size_t)S * kPoints, nout * sizeof(float),
                                        cudaMemcpyDeviceToHost, cs));
        LG_CUDA_TRY(cudaMemcpyAsync(h + err_off, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, cs));
        LG_CUDA_TRY(cudaEventRecord(c->pl_d2h[j % R], cs));
        return LG_OK;
    };
    auto collect = [&](int j) -> int {
        const int nb = nb_of(j), b0 = sb[j];
        LG_CUDA_TRY(cudaEventSynchronize(c->pl_d2h[j % R]));
        const float *h = hout(j);
        int herr = 0;
        std::memcpy(&herr, h + err_off, sizeof(int));
        if (herr) {
            lg_set_error("kernel reported error status %d", herr);
            return LG_ERR_DEVICE;
        }
        if (n.d.value_head) {
            std::memcpy(value + b0, h, (size_t)nb * sizeof(float));
        } else {
            std::memcpy(probs + (size_t)b0 * kPoints, h, (size_t)nb * kPoints * sizeof(float));
            if (want_logits)
                std::memcpy(logits + (size_t)b0 * kPoints, h + (size_t)S * kPoints,
                            (size_t)nb * kPoints * sizeof(float));
        }
        return LG_OK;
    };
    // super-chunk j + 1 is staged before j is launched (its slot last held
    // j + 1 - R, handed out by then), and j - 1 is handed out while j runs
    int rc = stage_in(0);
    int collected = 0;
    for (int j = 0; j < nsup && !rc; ++j) {
        if (j + 1 < nsup) {
            while (!rc && collected <= j + 1 - R) rc = collect(collected++);
            if (!rc) rc = stage_in(j + 1);
        }
        if (!rc) rc = launch(j);
        while (!rc && collected < j) rc = collect(collected++);
    }
    while (!rc && collected < nsup) rc = collect(collected++);
    if (rc) {
        // nothing may still use the slots or buffers when the call returns
        cudaStreamSynchronize(s);
        cudaStreamSynchronize(cs);
        if (rc == LG_ERR_DEVICE) cudaMemset(c->d_err, 0, sizeof(int));
        cudaGetLastError();
    }
    return rc;
}

// Host call: chunks of up to max_batch positions go through a cached CUDA
// graph of copy-in + forward + copy-out (one graph per chunk size and
// staging slot).  Two pinned slots alternate, so the host packs chunk k+1
// while the GPU runs chunk k; chunk k-2's results are handed back first.
// With `squares` / `to_move` (and `moves` for nets reading planes 24..31)
// instead of planes, each chunk copies in the boards (362 bytes a position,
// 16 more with moves) and the graph gathers the input planes on
// the GPU before the forward.
int run_host(lg_ctx *c, int net, const uint8_t *planes, int B, float T, float *probs,
             float *logits, float *value, const int8_t *squares = nullptr,
             const int8_t *to_move = nullptr, const int32_t *moves = nullptr) {
    Net &n = c->nets[net];
    if (!n.present) {
        lg_set_error("net %d was not created", net);
        return LG_ERR_ARG;
    }
    const bool boards = squares != nullptr;
    if (B < 0 || (B > 0 && !planes && !(squares && to_move))) {
        lg_set_error("bad batch");
        return LG_ERR_ARG;
    }
    if (boards && (n.d.c_in > kGatherPlanes || c->planes_c < 2)) {
        lg_set_error("board input gathers planes 0..%d; the net reads %d planes", kGatherPlanes - 1,
                     n.d.c_in);
        return LG_ERR_ARG;
    }
    const bool with_moves = boards && n.d.c_in > 24;
    // tensor-core nets: the gather writes the first layer's input rows, except
    // for chunks the small-batch kernel takes (it reads planes)
    const bool l5_boards = boards && n.d.precision != LG_FP32;
    if (with_moves && !moves && B > 0) {
        lg_set_error("the net reads planes 24..31 (ladders, ko, last moves, komi): moves are needed");
        return LG_ERR_ARG;
    }
    int rc = check_fault(c);
    if (rc) return rc;
    cudaSetDevice(c->device);
    if (l5_boards && B > c->max_batch && c->max_batch <= kPipeMaxBatch && !use_lat(c, n, c->max_batch) &&
        c->stall_kind < 0)
        return run_host_boards_pipe(c, net, B, T, probs, logits, value, squares, to_move, moves);
    const size_t per_in = (size_t)n.d.c_in * kPoints;
    const bool want_logits = logits != nullptr && !n.d.value_head;
    uint32_t tbits;
    std::memcpy(&tbits, &T, 4);
    uint8_t *hp[2] = {c->h_planes, c->h_planes_b};
    float *ho[2] = {c->h_out, c->h_out_b}, *hl[2] = {c->h_out2, c->h_out2_b};
    struct Pending {
        int b0 = 0, nb = 0;
        bool live = false;
    } pend[2];
    auto finish = [&](int slot) -> int {
        Pending &q = pend[slot];
        if (!q.live) return LG_OK;
        q.live = false;
        LG_CUDA_TRY(cudaEventSynchronize(c->host_done[slot]));
        int herr = 0;
        LG_CUDA_TRY(cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost));
        if (herr) {
            cudaMemset(c->d_err, 0, sizeof(int));
            lg_set_error("kernel reported error status %d", herr);
            return LG_ERR_DEVICE;
        }
        if (n.d.value_head) {
            std::memcpy(value + q.b0, ho[slot], (size_t)q.nb * sizeof(float));
        } else {
            std::memcpy(probs + (size_t)q.b0 * kPoints, ho[slot], (size_t)q.nb * kPoints * sizeof(float));
            if (want_logits)
                std::memcpy(logits + (size_t)q.b0 * kPoints, hl[slot], (size_t)q.nb * kPoints * sizeof(float));
        }
        return LG_OK;
    };
    int k = 0;
    for (int b0 = 0; b0 < B; b0 += c->max_batch, ++k) {
        const int slot = k & 1;
        const int nb = std::min(c->max_batch, B - b0);
        if ((rc = finish(slot))) {
            finish(slot ^ 1);
            return rc;
        }
        // boards: squares, to_move, then the moves at a 4-byte boundary
        const size_t mv_off = ((size_t)nb * (kPoints + 1) + 3) & ~(size_t)3;
        const size_t in_bytes = !boards ? (size_t)nb * per_in
                                        : (with_moves ? mv_off + (size_t)nb * 16 : (size_t)nb * (kPoints + 1));
        if (boards) {
            std::memcpy(hp[slot], squares + (size_t)b0 * kPoints, (size_t)nb * kPoints);
            std::memcpy(hp[slot] + (size_t)nb * kPoints, to_move + b0, (size_t)nb);
            if (with_moves) std::memcpy(hp[slot] + mv_off, moves + (size_t)b0 * 4, (size_t)nb * 16);
        } else {
            std::memcpy(hp[slot], planes + (size_t)b0 * per_in, in_bytes);
        }
        const bool l5_direct = l5_boards && !use_lat(c, n, nb);
        auto key = std::make_tuple(net, nb, n.d.value_head ? 0u : tbits,
                                   (want_logits ? 1 : 0) + 8 * slot + (boards ? 16 : 0));
        auto it = c->graphs.find(key);
        // an armed stall (lg_inject_stall) runs this chunk outside the graph
        // cache, so that no cached graph keeps the stalled launch
        const bool direct = c->stall_kind >= 0;
        if (direct || it == c->graphs.end()) {
            cudaGraph_t g;
            if (!direct) LG_CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            int nl = 0;
            if (boards) {
                cudaMemcpyAsync(c->d_boards, hp[slot], in_bytes, cudaMemcpyHostToDevice, c->stream);
                const int8_t *dsq = c->d_boards, *dtm = c->d_boards + (size_t)nb * kPoints;
                const int32_t *dmv = with_moves ? reinterpret_cast<const int32_t *>(c->d_boards + mv_off) : nullptr;
                const int which = net == LG_NET_POLICY ? 0 : 1;
                // tensor-core nets: the gather writes the first layer's
                // expanded input rows itself (no planes, no packing pass)
                rc = l5_direct ? launch_gather_l5(dsq, dtm, dmv, nb, which, n.d.c_in, n.tc[0].halves,
                                                  n.d.precision == LG_FP16, c->l5, c->stream)
                               : launch_gather(dsq, dtm, dmv, nb, which, n.d.c_in, c->d_planes, c->stream);
                nl = 1;
            } else {
                cudaMemcpyAsync(c->d_planes, hp[slot], in_bytes, cudaMemcpyHostToDevice, c->stream);
            }
            int nf = 0;
            if (!rc)
                rc = forward(c, net, c->d_planes, nb, T, c->d_probs, want_logits ? c->d_logits : nullptr,
                             c->d_value, c->stream, &nf, false, l5_direct);
            nl += nf;
            if (n.d.value_head) {
                cudaMemcpyAsync(ho[slot], c->d_value, (size_t)nb * sizeof(float), cudaMemcpyDeviceToHost,
                                c->stream);
            } else {
                cudaMemcpyAsync(ho[slot], c->d_probs, (size_t)nb * kPoints * sizeof(float),
                                cudaMemcpyDeviceToHost, c->stream);
                if (want_logits)
                    cudaMemcpyAsync(hl[slot], c->d_logits, (size_t)nb * kPoints * sizeof(float),
                                    cudaMemcpyDeviceToHost, c->stream);
            }
            if (direct) {
                if (rc) {
                    finish(slot ^ 1);
                    return rc;
                }
                c->launches += nl;
            } else {
                cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
                if (rc) {
                    if (ce == cudaSuccess) cudaGraphDestroy(g);
                    finish(slot ^ 1);
                    return rc;
                }
                LG_CUDA_TRY(ce);
                cudaGraphExec_t ge;
                cudaError_t ie = cudaGraphInstantiate(&ge, g, 0);
                cudaGraphDestroy(g);
                LG_CUDA_TRY(ie);
                it = c->graphs.emplace(key, std::make_pair(ge, nl)).first;
            }
        }
        if (!direct) {
            LG_CUDA_TRY(cudaGraphLaunch(it->second.first, c->stream));
            c->launches += it->second.second;
        }
        LG_CUDA_TRY(cudaEventRecord(c->host_done[slot], c->stream));
        pend[slot].b0 = b0;
        pend[slot].nb = nb;
        pend[slot].live = true;
    }
    // hand back the last two chunks in order
    const int last = (k - 1) & 1;
    if ((rc = finish(last ^ 1))) {
        finish(last);
        return rc;
    }
    return finish(last);
}

int run_device(lg_ctx *c, int net, const uint8_t *planes, int B, float T, float *probs,
               float *logits, float *value, cudaStream_t s) {
    Net &n = c->nets[net];
    if (!n.present) {
        lg_set_error("net %d was not created", net);
        return LG_ERR_ARG;
    }
    int rc = check_fault(c);
    if (rc) return rc;
    cudaSetDevice(c->device);
    size_t per_in = (size_t)n.d.c_in * kPoints;
    // Tensor-core nets: the finish launch of chunk k also packs chunk k+1's
    // planes (when neither chunk runs on the small-batch kernel), so a chunk
    // costs a trunk launch and a finish launch; chunks alternate between the
    // two first-layer buffers.  Trunk and finish are programmatic dependents
    // of the kernel before them: the trunk's prologue overlaps the previous
    // finish, and the next chunk's packing CTAs start on the SMs the trunk
    // leaves.  Every kernel that reads another's results waits for it
    // (griddepcontrol.wait), and each trunk signals its dependents only
    // after its own wait, so a packing CTA of chunk k's finish starts only
    // after chunk k-1's trunk -- the last reader of its buffer -- completed.
    const bool tc = n.d.precision != LG_FP32;
    bool l5_ready = false;
    int k = 0;
    for (int b0 = 0; b0 < B; b0 += c->max_batch, ++k) {
        int nb = std::min(c->max_batch, B - b0);
        const int nb1 = std::min(c->max_batch, B - b0 - nb);
        __nv_bfloat16 *const l5cur = (k & 1) ? c->l5b : c->l5, *const l5nxt = (k & 1) ? c->l5 : c->l5b;
        PackJob pk{};
        const PackJob *next = nullptr;
        if (tc && nb1 > 0 && (l5_ready || !use_lat(c, n, nb)) && !use_lat(c, n, nb1)) {
            pk.planes = planes + (size_t)(b0 + nb) * per_in;
            pk.B = nb1;
            pk.C = n.d.c_in;
            pk.halves = n.tc[0].halves;
            pk.f16 = n.d.precision == LG_FP16 ? 1 : 0;
            pk.out = l5nxt;
            next = &pk;
        }
        int nl = 0;
        rc = forward(c, net, planes + (size_t)b0 * per_in, nb, T,
                     probs ? probs + (size_t)b0 * kPoints : nullptr,
                     logits ? logits + (size_t)b0 * kPoints : nullptr, value ? value + b0 : nullptr,
                     s, &nl, c->profiling, l5_ready, next, l5cur, tc);
        l5_ready = next != nullptr;
        if (rc) return rc;
        c->launches += nl;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            lg_set_error("launch failed: %s", cudaGetErrorString(e));
            return LG_ERR_CUDA;
        }
    }
    return LG_OK;
}

// ------------------------------------------------------------ batching server
//
// Requests are taken in arrival order and packed into a batch of up to
// max_batch positions of one net (and, for the policy, one temperature); the
// batch is padded up to the next power of two so that a handful of CUDA
// graphs (one per bucket) serve every size.

int next_pow2(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

// Launches one server batch whose planes are already in pinned slot `slot`:
// a CUDA graph per (net, bucket, temperature, slot) holding the copy in, the
// forward and the copy out; completion is recorded on srv_done[slot].
// `net` may be LG_NET_POLICY_LOGITS: the policy net, head outputs copied out.
int server_launch(lg_ctx *c, int slot, int net, int nb, float T) {
    const bool logits = net == LG_NET_POLICY_LOGITS;
    Net &n = c->nets[logits ? LG_NET_POLICY : net];
    const size_t per_in = (size_t)n.d.c_in * kPoints;
    uint32_t tbits;
    std::memcpy(&tbits, &T, 4);
    auto key = std::make_tuple(net, nb, n.d.value_head ? 0u : tbits, 2 + slot);
    auto it = c->graphs.find(key);
    if (it == c->graphs.end()) {
        cudaGraph_t g;
        LG_CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        cudaMemcpyAsync(c->d_planes, c->srv_planes[slot], (size_t)nb * per_in, cudaMemcpyHostToDevice,
                        c->stream);
        int nl = 0;
        int rc = forward(c, logits ? LG_NET_POLICY : net, c->d_planes, nb, T, c->d_probs,
                         logits ? c->d_logits : nullptr, c->d_value, c->stream, &nl);
        if (n.d.value_head)
            cudaMemcpyAsync(c->srv_out[slot], c->d_value, (size_t)nb * sizeof(float), cudaMemcpyDeviceToHost,
                            c->stream);
        else
            cudaMemcpyAsync(c->srv_out[slot], logits ? c->d_logits : c->d_probs, (size_t)nb * kPoints * sizeof(float),
                            cudaMemcpyDeviceToHost, c->stream);
        cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
        if (rc) {
            if (ce == cudaSuccess) cudaGraphDestroy(g);
            return rc;
        }
        LG_CUDA_TRY(ce);
        cudaGraphExec_t ge;
        cudaError_t ie = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        LG_CUDA_TRY(ie);
        it = c->graphs.emplace(key, std::make_pair(ge, nl)).first;
    }
    LG_CUDA_TRY(cudaGraphLaunch(it->second.first, c->stream));
    LG_CUDA_TRY(cudaEventRecord(c->srv_done[slot], c->stream));
    c->launches += it->second.second;
    return LG_OK;
}

int server_finish(lg_ctx *c, int slot) {
    LG_CUDA_TRY(cudaEventSynchronize(c->srv_done[slot]));
    int herr = 0;
    LG_CUDA_TRY(cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) {
        cudaMemset(c->d_err, 0, sizeof(int));
        lg_set_error("kernel reported error status %d", herr);
        return LG_ERR_DEVICE;
    }
    return LG_OK;
}

// The server thread keeps at most two batches in flight: while batch k runs
// on the GPU it packs and launches batch k+1 into the other pinned slot,
// then waits for batch k and hands its results back.
void worker_main(lg_ctx *c) {
    cudaSetDevice(c->device);
    struct Flight {
        std::vector<lg_ctx::Req> reqs;
        int net = 0, slot = 0, rc = LG_OK;
        bool live = false;
    } fl[2];
    int next_slot = 0;
    for (;;) {
        std::vector<lg_ctx::Req> batch;
        bool have_inflight = fl[0].live || fl[1].live;
        {
            std::unique_lock<std::mutex> lk(c->qmu);
            if (!have_inflight) c->qcv.wait(lk, [&] { return c->stop || !c->queue.empty(); });
            if (c->stop && c->queue.empty() && !have_inflight) return;
            if (!c->queue.empty()) {
                // The oldest request picks the net (and temperature); every
                // queued request of that kind joins, in arrival order, while it fits.
                int total = 0;
                const int net = c->queue.front().net;
                const float T = c->queue.front().temperature;
                for (auto it = c->queue.begin(); it != c->queue.end();) {
                    const bool same = it->net == net && (net != LG_NET_POLICY || it->temperature == T);
                    if (!same) {
                        ++it;
                        continue;
                    }
                    if (total > 0 && total + it->B > c->max_batch) break;
                    total += it->B;
                    batch.push_back(*it);
                    it = c->queue.erase(it);
                }
            }
        }
        // Launch the new batch (if any) into the free slot.
        int launched = -1;
        if (!batch.empty()) {
            const int slot = fl[next_slot].live ? next_slot ^ 1 : next_slot;
            Flight &f = fl[slot];
            f.reqs = std::move(batch);
            f.net = f.reqs[0].net;
            f.slot = slot;
            Net &n = c->nets[f.net == LG_NET_VALUE ? LG_NET_VALUE : LG_NET_POLICY];
            const size_t per_in = (size_t)n.d.c_in * kPoints;
            int total = 0;
            for (auto &r : f.reqs) total += r.B;
            const int bucket = std::min(next_pow2(total), std::max(total, c->max_batch));
            size_t off = 0;
            for (auto &r : f.reqs) {
                std::memcpy(c->srv_planes[slot] + off, r.planes, (size_t)r.B * per_in);
                off += (size_t)r.B * per_in;
            }
            std::memset(c->srv_planes[slot] + off, 0, (size_t)(bucket - total) * per_in);
            {
                std::lock_guard<std::mutex> g(c->mu);
                f.rc = server_launch(c, slot, f.net, bucket, f.reqs[0].temperature);
            }
            f.live = true;
            launched = slot;
            next_slot = slot ^ 1;
            c->batches++;
        }
        // Finish the older batch in flight (not the one just launched), or the
        // only one when nothing new arrived.
        for (int k = 0; k < 2; ++k) {
            Flight &f = fl[k];
            if (!f.live || k == launched) continue;
            {
                int rc = f.rc;
                if (rc == LG_OK) {
                    std::lock_guard<std::mutex> g(c->mu);
                    rc = server_finish(c, f.slot);
                }
                const int per_out = f.net == LG_NET_VALUE ? 1 : kPoints;
                size_t o = 0;
                for (auto &r : f.reqs) {
                    if (rc == LG_OK)
                        std::memcpy(r.out, c->srv_out[f.slot] + o, (size_t)r.B * per_out * sizeof(float));
                    o += (size_t)r.B * per_out;
                }
                {
                    std::lock_guard<std::mutex> lk(c->qmu);
                    if (rc != LG_OK) c->worker_error = rc;
                    for (auto &r : f.reqs) c->done.push_back(r.tag);
                }
                c->dcv.notify_all();
                f.live = false;
                f.reqs.clear();
            }
        }
    }
}

// Device address of the static scratch array of lg_policy_device_static on
// `device` (current), resolved once per device and cached (defined below).
int static_scratch_resolve(int device, void **out);

}  // namespace

// ================================================================ C ABI

extern "C" size_t lg_weight_count(const lg_net_desc *desc) {
    if (!valid_desc(desc)) return 0;
    return weight_count(desc);
}

extern "C" void lg_destroy(lg_ctx *c) {
    if (!c) return;
    if (c->worker_started) {
        {
            std::lock_guard<std::mutex> lk(c->qmu);
            c->stop = true;
        }
        c->qcv.notify_all();
        c->worker.join();
    }
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto &g : c->graphs) cudaGraphExecDestroy(g.second.first);
    for (auto &t : c->prof_pending) {
        cudaEventDestroy(std::get<1>(t));
        cudaEventDestroy(std::get<2>(t));
    }
    for (auto e : c->event_pool) cudaEventDestroy(e);
    for (void *p : c->allocs) cudaFree(p);
    if (c->h_planes) cudaFreeHost(c->h_planes);
    if (c->h_out) cudaFreeHost(c->h_out);
    if (c->h_out2) cudaFreeHost(c->h_out2);
    if (c->h_planes_b) cudaFreeHost(c->h_planes_b);
    if (c->h_out_b) cudaFreeHost(c->h_out_b);
    if (c->h_out2_b) cudaFreeHost(c->h_out2_b);
    for (int i = 0; i < 2; ++i)
        if (c->host_done[i]) cudaEventDestroy(c->host_done[i]);
    if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
    for (int i = 0; i < lg_ctx::kPipe; ++i) {
        if (c->pl_h2d[i]) cudaEventDestroy(c->pl_h2d[i]);
        if (c->pl_comp[i]) cudaEventDestroy(c->pl_comp[i]);
        if (c->pl_d2h[i]) cudaEventDestroy(c->pl_d2h[i]);
    }
    if (c->pl_h_in) cudaFreeHost(c->pl_h_in);
    if (c->pl_h_out) cudaFreeHost(c->pl_h_out);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    for (int i = 0; i < 2; ++i) {
        if (c->srv_planes[i]) cudaFreeHost(c->srv_planes[i]);
        if (c->srv_out[i]) cudaFreeHost(c->srv_out[i]);
        if (c->srv_done[i]) cudaEventDestroy(c->srv_done[i]);
    }
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

extern "C" int lg_create(const lg_net_desc *policy, const lg_net_desc *value, int device,
                         int max_batch, lg_ctx **out) {
    if (!out || (!policy && !value) || max_batch < 1 || max_batch > (1 << 16)) {
        lg_set_error("lg_create: bad arguments");
        return LG_ERR_ARG;
    }
    *out = nullptr;
    if (policy && policy->value_head) {
        lg_set_error("policy description has value_head set");
        return LG_ERR_ARG;
    }
    if (value && !value->value_head) {
        lg_set_error("value description lacks value_head");
        return LG_ERR_ARG;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        lg_set_error("no CUDA device %d", device);
        return LG_ERR_CUDA;
    }
    lg_ctx *c = new lg_ctx();
    c->device = device;
    c->max_batch = max_batch;
    int rc = LG_OK;
    auto fail = [&](int r) {
        lg_destroy(c);
        return r;
    };
    if (cudaSetDevice(device) != cudaSuccess) return fail(LG_ERR_CUDA);
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(LG_ERR_CUDA);
    const lg_net_desc *descs[2] = {policy, value};
    size_t max_act = 0, max_partial = 0, max_tc_l3 = 0, max_tc_l5 = 0;
    int max_c_in = 0, max_fc = 0;
    for (int i = 0; i < 2; ++i) {
        if (!descs[i]) continue;
        if ((rc = build_net(c, c->nets[i], descs[i]))) return fail(rc);
        Net &n = c->nets[i];
        max_c_in = std::max(max_c_in, n.d.c_in);
        if (n.d.value_head) max_fc = std::max(max_fc, n.d.fc_hidden);
        if (n.d.precision == LG_FP32) {
            for (auto &s : n.shapes) {
                max_act = std::max(max_act, (size_t)std::max(s.cin, s.cout));
                for (int b = 1; b <= max_batch; b = (b < 64 ? b + 1 : b * 2))
                    max_partial = std::max(max_partial, conv_f32_partial_floats(b, s.cin, s.cout, s.k));
                max_partial = std::max(max_partial, conv_f32_partial_floats(max_batch, s.cin, s.cout, s.k));
            }
        } else {
            if ((rc = tc_init_device())) return fail(rc);
            max_tc_l3 = std::max(max_tc_l3, (size_t)n.d.width);
            max_tc_l5 = std::max(max_tc_l5, (size_t)n.tc[0].halves * 64);
        }
    }
    if ((rc = finish_init_device())) return fail(rc);
    size_t mb = (size_t)max_batch;
    if (max_act) {
        if ((rc = dev_alloc(c, &c->act[0], mb * kPoints * max_act)) ||
            (rc = dev_alloc(c, &c->act[1], mb * kPoints * max_act)) ||
            (rc = dev_alloc(c, &c->partial, max_partial)))
            return fail(rc);
    }
    if (max_tc_l3) {
        if ((rc = dev_alloc(c, &c->l3[0], mb * kL3Board * max_tc_l3)) ||
            (rc = dev_alloc(c, &c->l3[1], mb * kL3Board * max_tc_l3)) ||
            (rc = dev_alloc(c, &c->l5, mb * kL5Board * max_tc_l5)) ||
            (rc = dev_alloc(c, &c->l5b, mb * kL5Board * max_tc_l5)))
            return fail(rc);
        // Pad rows of the L3 buffers are read as zeros and never written
        // with anything else.
        if (cudaMemset(c->l3[0], 0, mb * kL3Board * max_tc_l3 * 2) != cudaSuccess ||
            cudaMemset(c->l3[1], 0, mb * kL3Board * max_tc_l3 * 2) != cudaSuccess)
            return fail(LG_ERR_CUDA);
    }
    bool any_lat = false;
    for (int i = 0; i < 2; ++i) any_lat |= c->nets[i].present && c->nets[i].lat_ok;
    if (any_lat) {
        if ((rc = lat_init_device()) || (rc = dev_alloc(c, &c->lat_part, lat_part_floats())) ||
            (rc = dev_alloc(c, &c->lat_cnt, (size_t)kLatCntInts)) ||
            (rc = dev_alloc(c, &c->lat_fcv, (size_t)kLatMaxB * kLatSplits)))
            return fail(rc);
        if (cudaMemset(c->lat_cnt, 0, sizeof(int) * kLatCntInts) != cudaSuccess) return fail(LG_ERR_CUDA);
    }
    default_tuning(c);
    // An FP32 policy net can be evaluated by lg_policy_device_static: look
    // up its static array's device address now, so that its calls only read
    // the cached pointer.
    if (policy && policy->precision == LG_FP32) {
        void *sp = nullptr;
        if ((rc = static_scratch_resolve(device, &sp))) return fail(rc);
    }
    c->planes_c = max_c_in;
    if ((rc = dev_alloc(c, &c->d_planes, mb * max_c_in * kPoints)) ||
        (rc = dev_alloc(c, &c->d_boards, mb * 384)) ||
        (rc = dev_alloc(c, &c->d_logits, mb * kPoints)) ||
        (rc = dev_alloc(c, &c->d_probs, mb * kPoints)) ||
        (rc = dev_alloc(c, &c->d_value, mb)) || (rc = dev_alloc(c, &c->d_err, 1)) ||
        (rc = dev_alloc(c, &c->d_parts, 4 * mb * kPoints)) ||
        (rc = dev_alloc(c, &c->d_fcpart, value_fc_part_floats(max_batch, std::max(max_fc, 1)))) ||
        (rc = dev_alloc(c, &c->d_fccnt, value_fc_counter_ints(max_batch, std::max(max_fc, 1)))) ||
        (rc = dev_alloc(c, &c->d_flags, trunk_flag_ints(max_batch * kL3Board, max_batch * kL5Board))))
        return fail(rc);
    // the counters and flags start at zero; every launch leaves them so
    if (cudaMemset(c->d_err, 0, sizeof(int)) != cudaSuccess ||
        cudaMemset(c->d_fccnt, 0, sizeof(int) * value_fc_counter_ints(max_batch, std::max(max_fc, 1))) != cudaSuccess ||
        cudaMemset(c->d_flags, 0, sizeof(int) * trunk_flag_ints(max_batch * kL3Board, max_batch * kL5Board)) !=
            cudaSuccess)
        return fail(LG_ERR_CUDA);
    if (cudaMallocHost(&c->h_planes, mb * max_c_in * kPoints) != cudaSuccess ||
        cudaMallocHost(&c->h_out, mb * kPoints * sizeof(float)) != cudaSuccess ||
        cudaMallocHost(&c->h_out2, mb * kPoints * sizeof(float)) != cudaSuccess ||
        cudaMallocHost(&c->h_planes_b, mb * max_c_in * kPoints) != cudaSuccess ||
        cudaMallocHost(&c->h_out_b, mb * kPoints * sizeof(float)) != cudaSuccess ||
        cudaMallocHost(&c->h_out2_b, mb * kPoints * sizeof(float)) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->host_done[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->host_done[1], cudaEventDisableTiming) != cudaSuccess) {
        lg_set_error("cudaMallocHost failed");
        return fail(LG_ERR_ALLOC);
    }
    for (int i = 0; i < 2; ++i) {
        if (cudaMallocHost(&c->srv_planes[i], mb * max_c_in * kPoints) != cudaSuccess ||
            cudaMallocHost(&c->srv_out[i], mb * kPoints * sizeof(float)) != cudaSuccess ||
            cudaEventCreateWithFlags(&c->srv_done[i], cudaEventDisableTiming) != cudaSuccess) {
            lg_set_error("cudaMallocHost failed");
            return fail(LG_ERR_ALLOC);
        }
    }
    if (cudaDeviceSynchronize() != cudaSuccess) {
        lg_set_error("device error after upload");
        return fail(LG_ERR_CUDA);
    }
    *out = c;
    return LG_OK;
}

extern "C" int lg_policy(lg_ctx *c, const uint8_t *planes, int B, float temperature, float *probs,
                         float *logits) {
    if (!c || !probs || !(temperature > 0.0f)) {
        lg_set_error("lg_policy: bad arguments");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(c->mu);
    return run_host(c, LG_NET_POLICY, planes, B, temperature, probs, logits, nullptr);
}

extern "C" int lg_value(lg_ctx *c, const uint8_t *planes, int B, float *value) {
    if (!c || !value) {
        lg_set_error("lg_value: bad arguments");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(c->mu);
    return run_host(c, LG_NET_VALUE, planes, B, 1.0f, nullptr, nullptr, value);
}

extern "C" int lg_policy_boards(lg_ctx *c, const int8_t *squares, const int8_t *to_move, const int32_t *moves,
                                int B, float temperature, float *probs, float *logits) {
    if (!c || !probs || !(temperature > 0.0f) || (B > 0 && (!squares || !to_move))) {
        lg_set_error("lg_policy_boards: bad arguments");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(c->mu);
    return run_host(c, LG_NET_POLICY, nullptr, B, temperature, probs, logits, nullptr, squares, to_move, moves);
}

extern "C" int lg_value_boards(lg_ctx *c, const int8_t *squares, const int8_t *to_move, const int32_t *moves,
                               int B, float *value) {
    if (!c || !value || (B > 0 && (!squares || !to_move))) {
        lg_set_error("lg_value_boards: bad arguments");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(c->mu);
    return run_host(c, LG_NET_VALUE, nullptr, B, 1.0f, nullptr, nullptr, value, squares, to_move, moves);
}

extern "C" int lg_policy_device(lg_ctx *c, const uint8_t *planes, int B, float temperature,
                                float *probs, float *logits, void *stream) {
    if (!c || !planes || !probs || B < 0 || !(temperature > 0.0f)) {
        lg_set_error("lg_policy_device: bad arguments");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(c->mu);
    return run_device(c, LG_NET_POLICY, planes, B, temperature, probs, logits, nullptr,
                      (cudaStream_t)stream);
}

extern "C" int lg_value_device(lg_ctx *c, const uint8_t *planes, int B, float *value,
                               void *stream) {
    if (!c || !planes || !value || B < 0) {
        lg_set_error("lg_value_device: bad arguments");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(c->mu);
    return run_device(c, LG_NET_VALUE, planes, B, 1.0f, nullptr, nullptr, value,
                      (cudaStream_t)stream);
}

// The learned fast path over B positions, all on `stream`: the student
// (fused kernel, softmax with entropy, value FC) answers every position; the
// gate compacts the indices of those above the entropy threshold; their
// planes are gathered and run through the full nets in chunks of max_batch
// whose sizes the kernels read from the device-side count; the full nets'
// answers are scattered over the student's.
extern "C" int lg_gated_device(lg_fast *f, lg_ctx *c, const uint8_t *planes_p, const uint8_t *planes_v, int B,
                               float temperature, float threshold, float *probs, float *value, uint8_t *fallback,
                               int32_t *count, void *stream) {
    if (!f || !c || !planes_p || !planes_v || (((uintptr_t)planes_p | (uintptr_t)planes_v) & 3) || B < 1 || !probs ||
        !value || !(temperature > 0.0f)) {
        lg_set_error("lg_gated_device: bad arguments (planes 4-byte aligned)");
        return LG_ERR_ARG;
    }
    Net &np = c->nets[LG_NET_POLICY], &nv = c->nets[LG_NET_VALUE];
    if (!np.present || !nv.present || np.d.precision == LG_FP32 || nv.d.precision == LG_FP32 ||
        !trunk_fusable(np) || !trunk_fusable(nv)) {
        lg_set_error("lg_gated_device: the full context needs tensor-core policy and value nets "
                     "(128 wide, 5x5 first layer)");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> lf(fast_mutex(f));
    std::lock_guard<std::mutex> lc(c->mu);
    cudaSetDevice(c->device);
    const size_t bytes_p = (size_t)np.d.c_in * kPoints, bytes_v = (size_t)nv.d.c_in * kPoints;
    GateScratch g{};
    int rc = fast_gate_scratch(f, bytes_p, bytes_v, &g);
    if (rc) return rc;
    if (B > g.max_batch || g.device != c->device || g.c_in != np.d.c_in || bytes_p % 4 || bytes_v % 4) {
        lg_set_error("lg_gated_device: B above the student's max_batch, another device, or the student's "
                     "input planes differ from the policy net's");
        return LG_ERR_ARG;
    }
    rc = check_fault(c);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    int nl = 0;
    long long total = 0;
    rc = fast_forward(f, planes_p, B, temperature, probs, nullptr, value, g.entropy, s, &nl);
    if (rc) return rc;
    total += nl;
    launch_gate(g.entropy, B, threshold, fallback ? fallback : g.fallback, g.idx, g.count, count, s);
    launch_gate_gather(planes_p, (int)bytes_p, g.idx, g.count, B, g.planes_p, s);
    launch_gate_gather(planes_v, (int)bytes_v, g.idx, g.count, B, g.planes_v, s);
    total += 3;
    for (int b0 = 0; b0 < B; b0 += c->max_batch) {
        const int nb = std::min(c->max_batch, B - b0);
        rc = forward_tc(c, np, g.planes_p + (size_t)b0 * bytes_p, nb, temperature, g.probs + (size_t)b0 * kPoints,
                        nullptr, nullptr, s, &nl, c->profiling, false, g.count, b0);
        if (rc) return rc;
        total += nl;
        rc = forward_tc(c, nv, g.planes_v + (size_t)b0 * bytes_v, nb, 1.0f, nullptr, nullptr, g.value + b0, s, &nl,
                        c->profiling, false, g.count, b0);
        if (rc) return rc;
        total += nl;
    }
    launch_gate_scatter(g.probs, g.value, g.idx, g.count, B, probs, value, s);
    total += 1;
    c->launches += total;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        lg_set_error("lg_gated_device: launch failed: %s", cudaGetErrorString(e));
        return LG_ERR_CUDA;
    }
    return LG_OK;
}

extern "C" int lg_submit(lg_ctx *c, int net, const uint8_t *planes, int B, float temperature,
                         float *out, void *tag) {
    if (!c || net < LG_NET_POLICY || net > LG_NET_POLICY_LOGITS ||
        !c->nets[net == LG_NET_VALUE ? LG_NET_VALUE : LG_NET_POLICY].present || !planes || !out || B < 1 ||
        B > c->max_batch || !(temperature > 0.0f)) {
        lg_set_error("lg_submit: bad arguments");
        return LG_ERR_ARG;
    }
    {
        std::lock_guard<std::mutex> lk(c->qmu);
        if (c->worker_error) {
            int e = c->worker_error;
            c->worker_error = 0;
            lg_set_error("an earlier batch failed");
            return e;
        }
        if (!c->worker_started) {
            c->worker = std::thread(worker_main, c);
            c->worker_started = true;
        }
        c->queue.push_back({net, planes, B, temperature, out, tag});
    }
    c->qcv.notify_one();
    return LG_OK;
}

extern "C" int lg_poll(lg_ctx *c, void **tags, int max, int timeout_us) {
    if (!c || !tags || max < 1 || timeout_us < 0) {
        lg_set_error("lg_poll: bad arguments");
        return LG_ERR_ARG;
    }
    std::unique_lock<std::mutex> lk(c->qmu);
    if (c->done.empty() && timeout_us > 0)
        c->dcv.wait_for(lk, std::chrono::microseconds(timeout_us), [&] { return !c->done.empty(); });
    int n = 0;
    while (n < max && !c->done.empty()) {
        tags[n++] = c->done.front();
        c->done.pop_front();
    }
    if (n == 0 && c->worker_error) {
        int e = c->worker_error;
        c->worker_error = 0;
        lg_set_error("a batch failed");
        return e;
    }
    return n;
}

extern "C" int lg_stats(lg_ctx *c, long long *kernel_launches, long long *batches) {
    if (!c) return LG_ERR_ARG;
    if (kernel_launches) *kernel_launches = c->launches.load();
    if (batches) *batches = c->batches.load();
    return LG_OK;
}

extern "C" int lg_device_error(lg_ctx *c) {
    if (!c) return LG_ERR_ARG;
    std::lock_guard<std::mutex> g(c->mu);
    cudaSetDevice(c->device);
    int herr = 0;
    LG_CUDA_TRY(cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) {
        LG_CUDA_TRY(cudaMemset(c->d_err, 0, sizeof(int)));
        lg_set_error("kernel reported error status %d", herr);
        return LG_ERR_DEVICE;
    }
    return LG_OK;
}

extern "C" int lg_inject_fault(lg_ctx *c, int nth_call) {
    if (!c || nth_call < 0) return LG_ERR_ARG;
    c->fault_in = nth_call;
    return LG_OK;
}

extern "C" int lg_inject_stall(lg_ctx *c, int kind, int polls) {
    if (!c || kind < -1 || kind > 1 || polls < 0) {
        lg_set_error("lg_inject_stall: bad arguments");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(c->mu);
    c->stall_kind = kind;
    c->stall_polls = (uint32_t)(polls ? polls : 1 << 12);
    return LG_OK;
}

extern "C" int lg_profile(lg_ctx *c, int enable) {
    if (!c) return LG_ERR_ARG;
    std::lock_guard<std::mutex> g(c->mu);
    c->profiling = enable != 0;
    for (int k = 0; k < LG_PROF_KINDS; ++k) {
        c->prof_launches[k] = 0;
        c->prof_ms[k] = 0.0;
    }
    for (auto &t : c->prof_pending) {
        c->event_pool.push_back(std::get<1>(t));
        c->event_pool.push_back(std::get<2>(t));
    }
    c->prof_pending.clear();
    return LG_OK;
}

extern "C" int lg_profile_read(lg_ctx *c, int kind, long long *launches, double *total_ms) {
    if (!c || kind < 0 || kind >= LG_PROF_KINDS) {
        lg_set_error("lg_profile_read: bad arguments");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(c->mu);
    for (auto &t : c->prof_pending) {
        cudaEvent_t a = std::get<1>(t), b = std::get<2>(t);
        LG_CUDA_TRY(cudaEventSynchronize(b));
        float ms = 0.0f;
        LG_CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
        c->prof_launches[std::get<0>(t)] += 1;
        c->prof_ms[std::get<0>(t)] += ms;
        c->event_pool.push_back(a);
        c->event_pool.push_back(b);
    }
    c->prof_pending.clear();
    if (launches) *launches = c->prof_launches[kind];
    if (total_ms) *total_ms = c->prof_ms[kind];
    return LG_OK;
}

// ============================================================================
// FP32 policy forward with no allocation at call time.
//
// For callers that must not allocate device memory when they evaluate a
// position: a search thread inside a process whose device memory belongs to
// another allocator, code that must not hit cudaMalloc/cudaFree's implicit
// device synchronisation in its latency path, or a host callback where CUDA
// allocation calls are not allowed.  The conv layers' split-K partial sums,
// the two activation buffers and the logits live in one file-scope device
// array of kStaticScratchBytes, shared by every call on every context.
// ============================================================================

namespace {
constexpr size_t kStaticScratchBytes = 8u << 20;  // 8 MiB, held by every GPU that loads this library
constexpr int kStaticMaxBatch = 4;
constexpr int kStaticMaxDevices = 64;
std::mutex g_static_mu;
void *g_static_ptr[kStaticMaxDevices] = {};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
}  // namespace

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

namespace {
// Once per device, with that device current: the device address of the
// array (its name in host code is only a host-side stand-in).  Contexts with
// an FP32 policy net do this when they are created.
int static_scratch_resolve(int device, void **out) {
    if (device < 0 || device >= kStaticMaxDevices) {
        lg_set_error("static scratch: device %d out of range", device);
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(g_static_mu);
    if (!g_static_ptr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p) {
            lg_set_error("cudaGetSymbolAddress(static scratch): %s", cudaGetErrorString(e));
            return LG_ERR_CUDA;
        }
        g_static_ptr[device] = p;
    }
    *out = g_static_ptr[device];
    return LG_OK;
}
}  // namespace

extern "C" int lg_policy_device_static(lg_ctx *c, const uint8_t *planes, int B, float temperature,
                                       float *probs, float *logits, void *stream) {
    if (!c || !planes || !probs || !(temperature > 0.0f) || B < 0) {
        lg_set_error("lg_policy_device_static: bad arguments");
        return LG_ERR_ARG;
    }
    if (B > kStaticMaxBatch) {
        lg_set_error("lg_policy_device_static: batch %d exceeds the static scratch limit of %d positions",
                     B, kStaticMaxBatch);
        return LG_ERR_ARG;
    }
    Net &n = c->nets[LG_NET_POLICY];
    if (!n.present || n.d.precision != LG_FP32) {
        lg_set_error("lg_policy_device_static: needs an FP32 policy net");
        return LG_ERR_ARG;
    }
    if (B == 0) return LG_OK;
    int rc = check_fault(c);
    if (rc) return rc;
    // Scratch layout: activations x2, split-K partials, logits.
    size_t max_ch = (size_t)n.d.c_in, max_partial = 0;
    for (auto &sh : n.shapes) {
        max_ch = std::max(max_ch, (size_t)std::max(sh.cin, sh.cout));
        max_partial = std::max(max_partial, conv_f32_partial_floats(B, sh.cin, sh.cout, sh.k));
    }
    const size_t act_bytes = align256((size_t)B * kPoints * max_ch * sizeof(float));
    const size_t part_bytes = align256(max_partial * sizeof(float));
    const size_t logit_bytes = align256((size_t)B * kPoints * sizeof(float));
    const size_t need = 2 * act_bytes + part_bytes + logit_bytes;
    if (need > kStaticScratchBytes) {
        lg_set_error("lg_policy_device_static: this net needs %zu bytes of scratch at batch %d, the static "
                     "array holds %zu",
                     need, B, kStaticScratchBytes);
        return LG_ERR_ARG;
    }
    LG_CUDA_TRY(cudaSetDevice(c->device));
    // The address was resolved when the context was created (lg_create); a
    // lookup here happens only if that did not run.
    void *base = nullptr;
    if ((rc = static_scratch_resolve(c->device, &base))) return rc;
    unsigned char *b = static_cast<unsigned char *>(base);
    float *act[2] = {reinterpret_cast<float *>(b), reinterpret_cast<float *>(b + act_bytes)};
    float *partial = reinterpret_cast<float *>(b + 2 * act_bytes);
    float *lg = logits ? logits : reinterpret_cast<float *>(b + 2 * act_bytes + part_bytes);
    cudaStream_t s = (cudaStream_t)stream;
    const lg_net_desc &d = n.d;
    launch_pack_planes_f32(planes, B, d.c_in, act[0], s);
    long long nlaunch = 1;
    int cur = 0;
    const int ntrunk = (int)n.shapes.size() - 1;
    for (int l = 0; l < ntrunk; ++l) {
        auto sh = n.shapes[l];
        launch_conv_f32(act[cur], n.wt[l], n.bias[l], act[cur ^ 1], B, sh.cin, sh.cout, sh.k, d.act,
                        partial, s);
        nlaunch += conv_f32_partial_floats(B, sh.cin, sh.cout, sh.k) ? 2 : 1;
        cur ^= 1;
    }
    auto hs = n.shapes.back();
    launch_head_conv_f32(act[cur], n.head_w, n.head_b, B, hs.cin, hs.k, d.act_head, d.act, lg, s);
    HeadIn h{lg, 1, 0, 0.0f, 0, d.act, nullptr};
    launch_softmax(h, B, temperature, probs, s);
    c->launches += nlaunch + 2;  // + head conv, softmax
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        lg_set_error("lg_policy_device_static: launch failed: %s", cudaGetErrorString(e));
        return LG_ERR_CUDA;
    }
    return LG_OK;
}

// ============================================================================
// Autotuner: for every power-of-two batch bucket up to max_batch, time the
// tensor-core nets' forward with each kernel choice for the 3x3 layers and
// for the first layer (256-row transposed kernel or 128-row kernel), keep
// the fastest, and cache the table as JSON keyed by device name, SM count
// and net widths.  FP32 nets have nothing to tune.
// ============================================================================

namespace {

std::string tune_key(lg_ctx *c) {
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, c->device);
    char buf[512];
    snprintf(buf, sizeof buf, "%s|sm%d|p%d/%d/%d|v%d/%d/%d|mb%d", prop.name, c->sm_count,
             c->nets[0].present ? c->nets[0].d.precision : -1, c->nets[0].present ? c->nets[0].d.width : 0,
             c->nets[0].present ? c->nets[0].d.c_in : 0, c->nets[1].present ? c->nets[1].d.precision : -1,
             c->nets[1].present ? c->nets[1].d.width : 0, c->nets[1].present ? c->nets[1].d.c_in : 0,
             c->max_batch);
    return buf;
}

bool load_tuning(lg_ctx *c, const char *path) {
    FILE *f = fopen(path, "r");
    if (!f) return false;
    std::string text;
    char buf[4096];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, n);
    fclose(f);
    std::string key = "\"key\": \"" + tune_key(c) + "\"";
    if (text.find(key) == std::string::npos) return false;
    int table[17][2] = {};
    for (int b = 0; b <= 16; ++b) {
        char pat[64];
        snprintf(pat, sizeof pat, "\"%d\": [", 1 << b);
        size_t pos = text.find(pat);
        if (pos == std::string::npos) continue;
        int a = 0, d = 0;
        if (sscanf(text.c_str() + pos + strlen(pat), "%d, %d", &a, &d) != 2) return false;
        if (a < 0 || a > 4 || d < 0 || d > 1) return false;
        table[b][0] = a;
        table[b][1] = d;
    }
    std::memcpy(c->tc_variant, table, sizeof table);
    return true;
}

int save_tuning(lg_ctx *c, const char *path, const double (*ms)[8]) {
    std::string tmp = std::string(path) + ".tmp";
    FILE *f = fopen(tmp.c_str(), "w");
    if (!f) {
        lg_set_error("cannot write %s", tmp.c_str());
        return LG_ERR_ARG;
    }
    fprintf(f, "{\n \"key\": \"%s\",\n \"order\": \"[3x3 layers: 0 = 256-row transposed per layer, 1 = 128-row per layer, 2 = persistent trunk, 3 = persistent trunk with the first layer in it, 4 = the whole net in one small-batch launch (FP32 nets: 0 = per-layer kernels, 4 = small-batch); first layer: 0 = 256-row, 1 = 128-row]; ms_per_forward for (3x3, first) = (0,0) (1,0) (2,0) (0,1) (1,1) (2,1) (3,0) (4,0), 0 = not timed\",\n \"table\": {",
            tune_key(c).c_str());
    bool first = true;
    for (int b = 0; (1 << b) <= c->max_batch && b <= 16; ++b) {
        fprintf(f, "%s\n  \"%d\": [%d, %d]", first ? "" : ",", 1 << b, c->tc_variant[b][0],
                c->tc_variant[b][1]);
        first = false;
    }
    fprintf(f, "\n },\n \"ms_per_forward\": {");
    first = true;
    for (int b = 0; (1 << b) <= c->max_batch && b <= 16; ++b) {
        fprintf(f, "%s\n  \"%d\": [%.4f, %.4f, %.4f, %.4f, %.4f, %.4f, %.4f, %.4f]", first ? "" : ",", 1 << b,
                ms[b][0], ms[b][1], ms[b][2], ms[b][3], ms[b][4], ms[b][5], ms[b][6], ms[b][7]);
        first = false;
    }
    fprintf(f, "\n }\n}\n");
    fclose(f);
    if (rename(tmp.c_str(), path) != 0) {
        lg_set_error("cannot rename %s", tmp.c_str());
        return LG_ERR_ARG;
    }
    return LG_OK;
}

}  // namespace

extern "C" int lg_autotune(lg_ctx *c, const char *cache_path, int force) {
    if (!c) {
        lg_set_error("lg_autotune: bad arguments");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(c->mu);
    bool any_tc = false, any_lat = false;
    for (int i = 0; i < 2; ++i) {
        any_tc |= c->nets[i].present && c->nets[i].d.precision != LG_FP32;
        any_lat |= c->nets[i].present && c->nets[i].lat_ok;
    }
    if (!any_tc && !any_lat) return LG_OK;
    if (cache_path && !force && load_tuning(c, cache_path)) {
        for (auto &gr : c->graphs) cudaGraphExecDestroy(gr.second.first);
        c->graphs.clear();
        c->tuned = true;
        return LG_OK;
    }
    LG_CUDA_TRY(cudaSetDevice(c->device));
    cudaEvent_t e0, e1;
    LG_CUDA_TRY(cudaEventCreate(&e0));
    LG_CUDA_TRY(cudaEventCreate(&e1));
    LG_CUDA_TRY(cudaMemsetAsync(c->d_planes, 0, (size_t)c->max_batch * c->planes_c * kPoints, c->stream));
    double ms[17][8] = {};
    int rc = LG_OK;
    // (3x3, first) of timing slot v: the six per-layer / trunk pairs, the
    // trunk with the first layer in it, the small-batch kernel
    auto choice = [](int v, int &v3, int &v1) {
        v3 = v < 6 ? v % 3 : (v == 6 ? 3 : 4);
        v1 = v < 6 ? v / 3 : 0;
    };
    for (int b = 0; (1 << b) <= c->max_batch && b <= 16 && rc == LG_OK; ++b) {
        const int B = 1 << b;
        double best = 1e30;
        int best_v = 0;
        for (int v = 0; v < 8 && rc == LG_OK; ++v) {
            if (v == 7 && (B > kLatMaxB || !any_lat)) continue;
            if (!any_tc && v != 0 && v != 7) continue;  // FP32 nets: per-layer or small-batch
            choice(v, c->tc_variant[b][0], c->tc_variant[b][1]);
            const int reps = B >= 64 ? 5 : 20;
            float t = 0.0f;
            for (int it = 0; it < 2 + reps && rc == LG_OK; ++it) {
                if (it == 2) cudaEventRecord(e0, c->stream);
                for (int net = 0; net < 2 && rc == LG_OK; ++net) {
                    Net &n = c->nets[net];
                    if (!n.present) continue;
                    int nl = 0;
                    rc = forward(c, net, c->d_planes, B, 1.0f, c->d_probs, nullptr, c->d_value, c->stream, &nl);
                }
            }
            if (rc) break;
            cudaEventRecord(e1, c->stream);
            LG_CUDA_TRY(cudaEventSynchronize(e1));
            cudaEventElapsedTime(&t, e0, e1);
            ms[b][v] = t / reps;
            if (ms[b][v] < best) {
                best = ms[b][v];
                best_v = v;
            }
        }
        choice(best_v, c->tc_variant[b][0], c->tc_variant[b][1]);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int herr = 0;
    cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (rc == LG_OK && herr) {
        cudaMemset(c->d_err, 0, sizeof(int));
        lg_set_error("kernel reported error status %d during tuning", herr);
        rc = LG_ERR_DEVICE;
    }
    for (auto &gr : c->graphs) cudaGraphExecDestroy(gr.second.first);
    c->graphs.clear();
    if (rc != LG_OK) {
        default_tuning(c);
        return rc;
    }
    c->tuned = true;
    if (cache_path) return save_tuning(c, cache_path, ms);
    return LG_OK;
}

extern "C" int lg_tuning(lg_ctx *c, int B, int *variant_3x3, int *variant_first) {
    if (!c || B < 1) return LG_ERR_ARG;
    int bl = 0;
    while ((1 << bl) < B && bl < 16) ++bl;
    if (variant_3x3) *variant_3x3 = c->tc_variant[bl][0];
    if (variant_first) *variant_first = c->tc_variant[bl][1];
    return c->tuned ? 1 : 0;
}

extern "C" int lg_set_tuning(lg_ctx *c, int B, int variant_3x3, int variant_first) {
    if (!c || B < 1 || variant_3x3 < 0 || variant_3x3 > 4 || variant_first < 0 || variant_first > 1) {
        lg_set_error("lg_set_tuning: bad arguments");
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(c->mu);
    int bl = 0;
    while ((1 << bl) < B && bl < 16) ++bl;
    c->tc_variant[bl][0] = variant_3x3;
    c->tc_variant[bl][1] = variant_first;
    for (auto &gr : c->graphs) cudaGraphExecDestroy(gr.second.first);
    c->graphs.clear();
    return LG_OK;
}

// ============================================================================
// 8-symmetry ensemble (AVERAGE_ALL): B positions -> a batch of 8B rotated
// copies -> one forward -> un-rotate and average on the device.
// ============================================================================

namespace {
std::once_flag g_rot_once[64];
int g_rot_rc[64];

int ensure_rot_tables(lg_ctx *c) {
    if (c->device < 0 || c->device >= 64) return LG_ERR_ARG;
    std::call_once(g_rot_once[c->device], [&] { g_rot_rc[c->device] = ensemble_init_tables(); });
    return g_rot_rc[c->device];
}
}  // namespace

extern "C" int lg_policy_avg8_device(lg_ctx *c, const uint8_t *planes, int B, float temperature,
                                     float *probs, void *stream) {
    if (!c || !planes || !probs || B < 0 || !(temperature > 0.0f)) {
        lg_set_error("lg_policy_avg8_device: bad arguments");
        return LG_ERR_ARG;
    }
    Net &n = c->nets[LG_NET_POLICY];
    if (!n.present) {
        lg_set_error("no policy net");
        return LG_ERR_ARG;
    }
    if (B == 0) return LG_OK;
    if (8 * B > c->max_batch) {
        lg_set_error("lg_policy_avg8_device: 8 x %d positions exceed max_batch %d", B, c->max_batch);
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(c->mu);
    LG_CUDA_TRY(cudaSetDevice(c->device));
    int rc = ensure_rot_tables(c);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    launch_rotate8(planes, B, n.d.c_in, c->d_planes, s);
    int nl = 0;
    rc = forward(c, LG_NET_POLICY, c->d_planes, 8 * B, temperature, c->d_probs, nullptr, nullptr, s, &nl,
                 c->profiling);
    if (rc) return rc;
    launch_unrotate_avg8(c->d_probs, B, probs, s);
    c->launches += nl + 2;
    LG_CUDA_TRY(cudaGetLastError());
    return LG_OK;
}

extern "C" int lg_value_avg8_device(lg_ctx *c, const uint8_t *planes, int B, float *value, void *stream) {
    if (!c || !planes || !value || B < 0) {
        lg_set_error("lg_value_avg8_device: bad arguments");
        return LG_ERR_ARG;
    }
    Net &n = c->nets[LG_NET_VALUE];
    if (!n.present) {
        lg_set_error("no value net");
        return LG_ERR_ARG;
    }
    if (B == 0) return LG_OK;
    if (8 * B > c->max_batch) {
        lg_set_error("lg_value_avg8_device: 8 x %d positions exceed max_batch %d", B, c->max_batch);
        return LG_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(c->mu);
    LG_CUDA_TRY(cudaSetDevice(c->device));
    int rc = ensure_rot_tables(c);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    launch_rotate8(planes, B, n.d.c_in, c->d_planes, s);
    int nl = 0;
    rc = forward(c, LG_NET_VALUE, c->d_planes, 8 * B, 1.0f, nullptr, nullptr, c->d_value, s, &nl, c->profiling);
    if (rc) return rc;
    launch_avg8(c->d_value, B, value, s);
    c->launches += nl + 2;
    LG_CUDA_TRY(cudaGetLastError());
    return LG_OK;
}

// lg_kernels.h -- launchers of the leela_gb300 kernels (internal).
#pragma once
#include "../../include/leela_gpu.h"
#include "lg_common.cuh"

#include <cuda_fp16.h>

#include <mutex>

namespace lg {

__device__ __forceinline__ float act_fn(float v, int act) {
    // ELU exactly as the reference writes it: x > 0 ? x : exp(x) - 1.
    if (act == LG_ACT_ELU) return (v > 0.0f) ? v : (expf(v) - 1.0f);
    if (act == LG_ACT_RELU) return (v > 0.0f) ? v : 0.0f;
    return v;  // any other code: identity (used by the training kernels)
}

// One value rounded to nearest even in the operand type (FP16 when f16, else
// BF16), as its 16 bits.
__device__ __forceinline__ uint16_t round16(float v, bool f16) {
    return f16 ? __half_as_ushort(__float2half_rn(v)) : __bfloat16_as_ushort(__float2bfloat16_rn(v));
}

// ------------------------------------------------------------ FP32 path
int conv_f32_splits(int M, int O, int C, int k);
size_t conv_f32_partial_floats(int B, int C, int O, int k);
void launch_pack_planes_f32(const uint8_t *planes, int B, int C, float *out, cudaStream_t s);
void launch_conv_f32(const float *in, const float *wt, const float *bias, float *out, int B,
                     int C, int O, int k, int act, float *partial, cudaStream_t s);
void launch_head_conv_f32(const float *in, const float *wh, float bias, int B, int C, int k,
                          int do_act, int act, float *logits, cudaStream_t s);
// Input of the finish kernels: the head output of point (b, p) is
//   act_head?(sum_k parts[k * part_stride + b * 361 + p] + head_b).
// When logits_out is set the finish kernel also writes that value there.
// With `count` set, only boards b < *count - count_base (read on the device)
// are processed: the batch size of a launch whose positions were selected
// on the device.
struct HeadIn {
    const float *parts;
    int nparts;
    size_t part_stride;
    float head_b;
    int head_act;
    int act;
    float *logits_out;
    const int *count = nullptr;
    int count_base = 0;
};
// entropy (optional): -sum p ln p of each board's probabilities, in nats.
// pdl: launched as a programmatic dependent of the previous kernel (the
// finish kernels wait for it before reading anything).
void launch_softmax(const HeadIn &h, int B, float temperature, float *probs, cudaStream_t s,
                    float *entropy = nullptr, bool pdl = false);
// Value head, one launch (tiled split-K FC1 pre-activations; the CTAs that
// finish last add them in a fixed order and run b1, the activation, FC2 and
// the value map); `part` holds value_fc_part_floats(B, H) floats, `cnt`
// value_fc_counter_ints(B, H) ints that are zero before the first launch
// (each launch leaves them zero).  w1s is W1 sliced by
// value_fc_slice_units() hidden units: [ceil(H/64)][361][64], zero-padded.
void launch_value_fc(const HeadIn &h, int B, const float *w1s, const float *b1, const float *w2,
                     float b2, int H, int act, int value_map, float *value, float *part, int *cnt,
                     cudaStream_t s, bool pdl = false);
size_t value_fc_part_floats(int B, int H);
// Kernel attributes of the finish kernels (once per device, before the first
// launch on it).
int finish_init_device();
size_t value_fc_counter_ints(int B, int H);
int value_fc_slice_units();

// The finish of one batch (softmax, or the value head as launch_value_fc)
// and the packing of the next batch's planes into the L5 rows
// (launch_pack_planes_l5's output) in one launch; the two touch disjoint
// memory.
struct FinishJob {
    HeadIn h;
    int B;
    int value_head;
    float temperature;  // policy
    float *probs, *entropy;
    const float *w1s, *b1, *w2;  // value
    float b2;
    int H, act, value_map;
    float *value, *part;
    int *cnt;
};
struct PackJob {
    const uint8_t *planes;  // [B][C][361]
    int B, C, halves, f16;
    __nv_bfloat16 *out;
};
// (For a value head these are two launches: the packing, then the head.)
// With pdl the launch is a programmatic dependent of the previous kernel
// (the batch's trunk): the packing CTAs run as soon as they are scheduled --
// `pk.out` must then be rows that kernel does not read -- and the finishing
// CTAs wait for it.
void launch_finish_pack(const FinishJob &j, const PackJob &pk, cudaStream_t s, bool pdl = false);

// ------------------------------------------------- tensor-core (tcgen05) path
//
// One conv layer as a persistent implicit GEMM on tcgen05: rows = flat
// activation rows (L3 or L5 layout), N = output channels, K = taps x input
// channels.  See tc_conv.cu.
struct TcLayer {
    const void *in;       // activations: [rows][cin_halves*64] BF16 (L3 or L5 rows)
    const void *w;        // weights: [taps][cin_halves][n][64] BF16
    const float *bias;    // [n]
    const float *scale;   // [n] per-output-channel weight scale (FP8 weights), or null
    const float *head_w;  // [n] fused 1x1 head weights (last trunk layer), or null;
                          // the fused head writes raw channel sums (no bias)
    int act;              // LG_ACT_*
    int cin_halves;       // input channels / 64
    int n;                // output channels (64 or 128)
    int in_kind;          // 0: L3 input (3x3); 1: L5 input (expanded 5x5 first layer)
    int rows;             // input rows processed (B * 400 or B * 399)
    int variant;          // for n == 128: 0 = 256-row transposed kernel, 1 = 128-row kernel
    int f16 = 0;          // activations and weights are FP16 (else BF16)
};

// Input planes 0..nplanes-1 (nplanes <= kGatherPlanes) of the policy
// (which = 0) or value (which = 1) set from boards: squares [B][361]
// (0 black, 1 white, 2 empty), to_move [B], moves [B][4] (last move, the
// move before it, ko point, white-has-komi flag; needed for planes 24..31);
// planes [B][nplanes][361].
constexpr int kGatherPlanes = 32;
// pdl: launched as a programmatic dependent of the previous kernel (a trunk):
// it gathers while that kernel's CTAs leave -- its output must be rows that
// kernel does not read -- and waits for it before exiting.
int launch_gather(const int8_t *squares, const int8_t *to_move, const int32_t *moves, int B, int which,
                  int nplanes, uint8_t *planes, cudaStream_t s, bool pdl = false);
// The same planes written straight as the first layer's expanded input (the
// rows launch_pack_planes_l5 makes from them, `halves` x 64 channels).
// (BF16 rows, or FP16 when f16.)
int launch_gather_l5(const int8_t *squares, const int8_t *to_move, const int32_t *moves, int B, int which,
                     int nplanes, int halves, bool f16, __nv_bfloat16 *l5, cudaStream_t s, bool pdl = false);

// Expanded 5x5 input: planes [B][C][361] bytes -> L5 rows (BF16, or FP16
// when f16) with halves*64 channels: channel dx*C + c = plane c at
// (y, x + dx - 2).
// With count set, boards b >= *count - count_base are skipped.
// With pdl the launch is a programmatic dependent of the previous kernel (a
// trunk): it packs without waiting for it (`out` must be rows it does not
// read) and waits for it before exiting.
void launch_pack_planes_l5(const uint8_t *planes, int B, int C, int halves, bool f16, __nv_bfloat16 *out,
                           cudaStream_t s, const int *count = nullptr, int count_base = 0, bool pdl = false);
// Writes the layer output (L3 rows) or, for the fused head, the head output
// before its bias into parts[boards*361] (tc_head_parts() = 1 array).
// Returns LG_ERR_ARG if no kernel covers the shape.
int launch_tc_conv(const TcLayer &L, __nv_bfloat16 *out_l3, float *parts, size_t part_stride,
                   int *err, cudaStream_t s, int sm_count);
int tc_head_parts(int n, int variant = 0);

// All 3x3 128->128 layers of a net in one persistent, cooperative launch
// (tc_trunk_kernel), scheduled as (layer, 256-row chunk) items claimed in
// order: layer l reads buf_a when l is even and buf_b when odd, and writes
// the other; the last layer writes head partial sums (4 parts) when head_w
// is set.
// With buf5 set, the 5x5 first layer (L5 input rows5 = B * 399, weights
// [5][2][128][64]) runs in the same launch as its own work items and writes
// buf_a.
struct TcTrunk {
    const void *buf_a, *buf_b;  // L3 activation buffers [rows][128] BF16
    const void *w;              // [nl][9][2][128][64] BF16
    const float *bias;          // [nl][128]
    const float *scale;         // [nl][128] or null
    const float *head_w;        // [128] or null
    int act;
    int rows;
    int nl;
    const void *buf5 = nullptr;  // fused first layer: L5 rows [rows5][128] BF16
    const void *w0 = nullptr;    // [5][2][128][64] BF16
    const float *bias0 = nullptr, *scale0 = nullptr;
    int rows5 = 0;
    int f16 = 0;                 // activations and weights are FP16 (else BF16)
    // wait limits (0: the defaults) and the test hook that makes one item
    // wait for a flag that nothing publishes (-1: none)
    uint32_t wait_limit = 0, poll_limit = 0;
    int stall_item = -1;
    // device-side batch size: with count set, only the first
    // *count - count_base boards of the rows are computed (rows and rows5
    // give the buffers' extent)
    const int *count = nullptr;
    int count_base = 0;
    // launched as a programmatic dependent of the previous kernel in the
    // stream (its prologue overlaps that kernel), instead of cooperatively
    bool pdl = false;
};
// flags: trunk_flag_ints(rows, rows5) ints of device scratch, zero before the first
// launch; the launch's last CTA leaves them zero again (no memset between launches).
int launch_tc_trunk(const TcTrunk &T, float *parts, size_t part_stride, int *flags, int *err,
                    cudaStream_t s, int sm_count);
size_t trunk_flag_ints(int rows, int rows5);
// index of the first work item of 3x3 layer k (rows5 = 0: no fused first layer)
int trunk_layer_item(int rows, int rows5, int k);
size_t tc_conv_smem_bytes(int n, int ntaps, int cin_halves);
int tc_init_device();
// Head kernels for the tensor-core path (logits already produced by the
// fused epilogue): same softmax / value FC as FP32.

// ------------------------------------------- small-batch path (latency.cu)
//
// Every conv layer of a net (the head as a layer of one output channel) in
// one cooperative launch for 1..kLatMaxB positions: units (board row, input
// channel split) of 8 splits a layer, partial sums per split in FP32, added
// by the consumer in a fixed order.  Weights per layer and split (input
// channels s*cg .. s*cg + cg - 1): FP32 [cg][k*k][cout], or for the 16-bit
// layers of tensor-core nets [9][128][16]; each split's block padded to
// `slice` floats (a multiple of 4).
constexpr int kLatMaxB = 8;
constexpr int kLatSplits = 8;
constexpr int kLatMaxRows = kLatMaxB * kBoard;
constexpr int kLatMaxLayers = 16;
constexpr int kLatMaxCg = 16;
constexpr int kLatSliceMax = 16 * 9 * 128;  // floats of one split's weights
// counters: [layer][row], then one per board for the value head, then the
// exit counter
constexpr int kLatCntFc = kLatMaxLayers * kLatMaxRows;
constexpr int kLatCntExit = kLatCntFc + kLatMaxB;
constexpr int kLatCntInts = kLatCntExit + 1;

struct LatConv {
    const void *w;       // [8][slice floats]: FP32 [cg][k*k][cout], or for 16-bit
                         // layers [9][cout = 128][16] BF16 / FP16
    const float *bias;   // [cout] (the consumer adds it)
    const float *scale;  // [cout] per-output-channel weight scale (FP8 weights), or null
    int k, cin, cout, cg, slice;
    int mma;             // 16-bit layer on the warp MMA (3x3, cg 16, cout 128)
};
struct LatParams {
    LatConv L[kLatMaxLayers];  // conv layers, then the head (cout 1)
    int nl;                    // conv layers + head
    int B, c_in, act, act_head;
    float head_b;
    const uint8_t *planes;     // [B][c_in][361]
    float *part;               // lat_part_floats()
    int *cnt;                  // kLatCntInts, zero between launches
    int *err;
    // policy: softmax
    float temperature;
    float *probs, *logits_out;
    // value: FC (w1s sliced [H/64][361][64]) + tanh / (1 + tanh) / 2
    int value_head;
    const float *w1s, *b1, *w2;
    float b2;
    int H, value_map;
    float *value;
    float *fcv;                // [kLatMaxB][8]
    uint32_t poll_limit;       // polls of one row counter before it gives up
    int stall_row;             // test hook: this layer-1 row waits for a count no unit reaches (-1: none)
};
size_t lat_part_floats();
size_t lat_smem_bytes();
int lat_init_device();
int lat_grid(int B, int sm_count);
// mode 0: FP32 nets; 1 / 2: BF16 / FP16 activations on the layers marked mma
int launch_lat(const LatParams &p, int mode, int sm_count, cudaStream_t s);

// ------------------------------------------- distilled student (fast_net.cu)
//
// The fused BF16 student trunk + both 1x1 heads, then softmax (+ entropy)
// and the value FC: four launches for B positions.  The gate kernels pick the
// positions whose entropy is above a threshold, gather their planes, and put
// the full nets' answers back in place; all counts stay on the device.
struct GateScratch {
    uint8_t *planes_p, *planes_v;
    float *probs, *value, *entropy;
    int *idx, *count;
    uint8_t *fallback;
    int max_batch, device, c_in;
};
int fast_forward(lg_fast *f, const uint8_t *planes, int B, float T, float *probs, float *logits, float *value,
                 float *entropy, cudaStream_t s, int *nlaunch);
int fast_gate_scratch(lg_fast *f, size_t bytes_p, size_t bytes_v, GateScratch *g);
std::mutex &fast_mutex(lg_fast *f);
int fast_status_word(lg_fast *f);
int fast_init_device();
int launch_gate(const float *entropy, int B, float threshold, uint8_t *fallback, int *idx, int *count,
                int *count_out, cudaStream_t s);
int launch_gate_gather(const uint8_t *src, int bytes, const int *idx, const int *count, int B, uint8_t *dst,
                       cudaStream_t s);
int launch_gate_scatter(const float *fprobs, const float *fvalue, const int *idx, const int *count, int B,
                        float *probs, float *value, cudaStream_t s);

// 8-symmetry ensemble helpers (ensemble.cu).
int ensemble_init_tables();
void launch_rotate8(const uint8_t *in, int B, int C, uint8_t *out, cudaStream_t s);
void launch_unrotate_avg8(const float *probs, int B, float *avg, cudaStream_t s);
void launch_avg8(const float *v, int B, float *out, cudaStream_t s);

// Tensor-map encoding through the driver entry point (no -lcuda needed).
int encode_map_2d_bf16(CUtensorMap *map, const void *base, uint64_t inner, uint64_t rows,
                       uint32_t box_inner, uint32_t box_rows, bool swizzle128 = true);

}  // namespace lg

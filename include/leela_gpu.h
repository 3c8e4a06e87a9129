/*
 * leela_gpu.h -- C ABI of the GB300 evaluation path for Leela's policy and
 * value networks.
 *
 * The host side of the engine (its Network class, Network.h:23-88) calls
 * these functions in place of its BLAS / OpenCL backends.  No C++ exception
 * and no CUDA or torch type crosses this boundary: plain pointers and sizes
 * in, an int status out (0 = ok, < 0 = error; lg_last_error() gives the
 * message for the calling thread).
 *
 * Board geometry is fixed at 19x19 (Network.cpp:352-355).  Input planes are
 * bytes holding 0 or 1, [B][c_in][361], point index y*19+x, already rotated
 * by the caller as Network.cpp:765-773 does.
 */
#ifndef LEELA_GPU_H
#define LEELA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define LG_API __attribute__((visibility("default")))
#else
#define LG_API
#endif

#define LG_OK 0
#define LG_ERR_ARG -1      /* bad argument or unsupported shape */
#define LG_ERR_ALLOC -2    /* device or host allocation failed */
#define LG_ERR_CUDA -3     /* CUDA runtime error */
#define LG_ERR_TIMEOUT -4  /* a bounded wait ran out */
#define LG_ERR_DEVICE -5   /* a kernel reported an error status */

#define LG_FP32 0 /* plain FP32: the drop-in path */
#define LG_BF16 1 /* BF16 activations and weights, FP32 accumulate (tcgen05) */
#define LG_FP8W 2 /* E4M3 weights with per-output-channel FP32 scales, BF16 activations */
#define LG_FP16 3 /* FP16 activations and weights, FP32 accumulate (tcgen05, same rate as BF16) */

#define LG_ACT_ELU 0  /* x > 0 ? x : exp(x) - 1 (Network.cpp:382-383) */
#define LG_ACT_RELU 1

#define LG_NET_POLICY 0
#define LG_NET_VALUE 1
#define LG_NET_POLICY_LOGITS 2 /* lg_submit only: the policy net's head output
                                  (logits) instead of probabilities */

/* Network shape and weights.  Conv layers in order: 5x5 c_in -> width1;
 * n3x3 layers 3x3 (width1 ->) width -> width; head head_k x head_k width -> 1.
 * `act` follows every conv but the head, and the head too if act_head.
 * Value nets (value_head = 1) add FC 361 -> fc_hidden (+act) and FC
 * fc_hidden -> 1, then tanh (value_map 0), (1 + tanh) / 2 (value_map 1,
 * Network.cpp:735-737), or no map (value_map 2: the FC output itself, for
 * callers that apply their own, as the OpenCL backend's callers do,
 * Network.cpp:704-705).
 *
 * weights: one flat FP32 array, per conv W[O][C][k][k] then b[O] (the
 * reference's OIHW arrays conv1_w, conv1_b, ... in order,
 * Network.cpp:54-137), then for value nets W1[fc_hidden][361], b1, W2, b2.
 * The library copies what it needs; the caller keeps ownership.
 *
 * LG_BF16 / LG_FP16 / LG_FP8W need c_in <= 32, width1 == width, width in
 * {64, 128} and head_k == 1.  LG_FP16 keeps 10 mantissa bits against
 * BF16's 7 (its range ends at 65504). */
typedef struct lg_net_desc {
    int c_in;
    int width1;
    int width;
    int n3x3;
    int head_k;
    int act;
    int act_head;
    int value_head;
    int fc_hidden;
    int value_map;
    int precision;
    const float *weights;
} lg_net_desc;

typedef struct lg_ctx lg_ctx;

/* Weight files.  lg_weights_save writes n nets (description + flat weights,
 * an optional name of up to 15 characters each) with a checksum, through a
 * temporary file and a rename.  lg_weights_load reads net `index`: with
 * weights == NULL it only reports the description and *count_out (to size a
 * buffer); with a buffer of `capacity` floats it also copies the weights and
 * sets desc->weights to that buffer.  Returns the number of nets in the file,
 * or LG_ERR_ARG with a message (missing file, bad magic or version,
 * checksum mismatch, truncation, count that does not fit the shape).
 * Replaces: the compiled-in weight arrays of NN.cpp / NN128.cpp /
 * NNValue.cpp (declared at Network.cpp:54-137), whose concatenation in
 * declaration order is exactly the flat lg_net_desc array. */
LG_API int lg_weights_save(const char *path, const lg_net_desc *descs, const char *const *names, int n);
LG_API int lg_weights_load(const char *path, int index, lg_net_desc *desc, char *name16, float *weights,
                           size_t capacity, size_t *count_out);

/* Number of floats in the flat weight array of `desc`. */
LG_API size_t lg_weight_count(const lg_net_desc *desc);

/* Uploads the nets (either may be NULL) to `device` and sizes every buffer
 * for up to max_batch positions per call.
 * Replaces: Network::initialize (Network.cpp:201-235), i.e.
 * OpenCL_Network::push_convolve / push_innerproduct (OpenCL.h:66-87,
 * OpenCL.cpp:579-744) and the device pick in OpenCL::initialize
 * (OpenCL.cpp:764-908). */
LG_API int lg_create(const lg_net_desc *policy, const lg_net_desc *value, int device, int max_batch,
              lg_ctx **out);

/* Frees every resource of the context.  No reference counterpart (the
 * reference keeps its nets for the life of the process). */
LG_API void lg_destroy(lg_ctx *ctx);

/* Message of the last failed call on this thread ("" if none).
 * Replaces: cl::Error / std::runtime_error (OpenCL.cpp:665-669, 848-850). */
LG_API const char *lg_last_error(void);

/* Policy net over B positions, blocking.  probs [B][361] = softmax of the
 * head output at `temperature`, network order (the caller un-rotates with
 * rev_rotate_nn_idx and filters EMPTY points, Network.cpp:820-829);
 * logits [B][361] (optional, may be NULL) = the head output before the
 * softmax.  Host buffers.
 * Replaces: the forward + softmax of Network::get_scored_moves_internal
 * (Network.cpp:742-832), OpenCL_Network::forward (OpenCL.cpp:490-569) and
 * Network::softmax (Network.cpp:450-469). */
LG_API int lg_policy(lg_ctx *ctx, const uint8_t *planes, int B, float temperature, float *probs,
              float *logits);

/* Value net over B positions, blocking; value [B].  Host buffers.
 * Replaces: Network::get_value_internal (Network.cpp:676-740). */
LG_API int lg_value(lg_ctx *ctx, const uint8_t *planes, int B, float *value);

/* Device-resident variants: every pointer is device memory and the work is
 * enqueued on `stream` (a cudaStream_t, NULL = the legacy default stream);
 * the call returns without waiting.  B may exceed max_batch: chunks of
 * max_batch run back to back, each chunk's launches as programmatic
 * dependents of the previous kernel on `stream`.  The calls of one context
 * share its device buffers: calls whose work could overlap on the GPU (on
 * different streams, or a blocking call while a device call still runs)
 * must be ordered by the caller -- one stream per context, or a stream
 * synchronisation between them.  A kernel's device-side error is read with
 * lg_device_error. */
LG_API int lg_policy_device(lg_ctx *ctx, const uint8_t *planes, int B, float temperature, float *probs,
                     float *logits, void *stream);
LG_API int lg_value_device(lg_ctx *ctx, const uint8_t *planes, int B, float *value, void *stream);

/* Input planes from boards, on the GPU.  squares [B][361] (0 black, 1 white,
 * 2 empty; point y*19+x, the order the planes use), to_move [B] (0 black,
 * 1 white); planes [B][nplanes][361] bytes, nplanes <= 32.  which = 0 writes
 * planes 0..nplanes-1 of the policy set, which = 1 of the value set: stone
 * colours, liberties of each string, the liberties a stone of either colour
 * would have on each empty point after its captures (0 for a suicide), the
 * ladder reader's "ladder" and "ladder win" planes, the ko point, the last
 * two moves (policy set), white's komi and the third line -- bit-exact with
 * the reference gather.  moves [B][4] int32 (last move, the move before it,
 * ko point: point indices, -1 for none; white-has-komi flag 0/1) is read only
 * for planes 24..31 and may be NULL when nplanes <= 24.  Device pointers,
 * enqueued on `stream`; needs no context.
 * Replaces: Network::gather_features_policy (Network.cpp:883-1046) and
 * Network::gather_features_value (Network.cpp:1048-1201), which run on the
 * host. */
LG_API int lg_gather_device(const int8_t *squares, const int8_t *to_move, const int32_t *moves, int B,
                            int which, int nplanes, uint8_t *planes, void *stream);

/* Host-buffer policy / value evaluation from boards (same encoding as
 * lg_gather_device): copies 362 bytes a position to the device (378 with
 * moves), gathers the net's input planes there (for BF16 / FP8 nets straight
 * into the first layer's input rows), then runs the forward;
 * results as lg_policy / lg_value, bit for bit.  Calls of more than
 * max_batch positions on the tensor-core nets run as a pipeline of
 * super-chunks (copies in and out on a second stream, overlapping the
 * forward of the super-chunk before), chunked as lg_policy / lg_value chunk.
 * moves may be NULL when the net reads at most 24 planes.
 * Replaces: Network::get_scored_moves (Network.cpp:624-674) and
 * Network::get_value (Network.cpp:590-622) at the DIRECT rotation, gather
 * included. */
LG_API int lg_policy_boards(lg_ctx *ctx, const int8_t *squares, const int8_t *to_move, const int32_t *moves,
                            int B, float temperature, float *probs, float *logits);
LG_API int lg_value_boards(lg_ctx *ctx, const int8_t *squares, const int8_t *to_move, const int32_t *moves,
                           int B, float *value);

/* 8-symmetry ensemble, device pointers, enqueued on `stream`: each of the B
 * positions (planes [B][c_in][361], unrotated) is evaluated under all 8
 * symmetries as one batch of 8B (8B <= max_batch); policy results are
 * un-rotated and averaged to board order (probs [B][361]: the caller keeps
 * the EMPTY points, as Network.cpp:820-829 does), values averaged
 * (value [B]).  Replaces: the AVERAGE_ALL branches of get_scored_moves and
 * get_value (Network.cpp:642-654, 606-615), which run 8 sequential forwards. */
LG_API int lg_policy_avg8_device(lg_ctx *ctx, const uint8_t *planes, int B, float temperature,
                                 float *probs, void *stream);
LG_API int lg_value_avg8_device(lg_ctx *ctx, const uint8_t *planes, int B, float *value, void *stream);

/* Batching server.  lg_submit queues B positions for net LG_NET_POLICY,
 * LG_NET_VALUE or LG_NET_POLICY_LOGITS and returns at once; `out` (host,
 * [B][361] probabilities at `temperature`, [B] values, or [B][361] head
 * outputs before the softmax for callers that apply their own, as the
 * OpenCL backend's forward_cb does, Network.cpp:484-494) is filled before
 * `tag` is reported by lg_poll.  A worker thread gathers queued requests into batches of up to
 * max_batch, pads each batch to a power-of-two bucket and replays the CUDA
 * graph captured for that bucket.  lg_poll copies up to `max` completed tags
 * and returns how many, waiting at most timeout_us microseconds (0 = do not
 * wait).
 * Replaces: Network::async_scored_moves + forward_cb (Network.cpp:484-587)
 * and OpenCL::thread_can_issue / callback_finished / join_outstanding_cb
 * (OpenCL.cpp:446-577), whose final wait is unbounded; this one is bounded. */
LG_API int lg_submit(lg_ctx *ctx, int net, const uint8_t *planes, int B, float temperature, float *out,
              void *tag);
LG_API int lg_poll(lg_ctx *ctx, void **tags, int max, int timeout_us);

/* Counters of the context: kernel launches issued so far (graph replays
 * count their kernels), and batches served by the batching server. */
LG_API int lg_stats(lg_ctx *ctx, long long *kernel_launches, long long *batches);

/* Device-side error of the device-pointer calls (no counterpart in the
 * reference, whose OpenCL calls block).  lg_policy_device / lg_value_device
 * return without waiting, so a kernel whose bounded wait ran out (what a
 * blocking call reports as LG_ERR_DEVICE) only records a code in the
 * context's error word.  After synchronizing the streams it used, the caller
 * reads it here: LG_OK, or LG_ERR_DEVICE with the code in lg_last_error(),
 * and the word is cleared. */
LG_API int lg_device_error(lg_ctx *ctx);

/* FP32 policy forward that allocates nothing (no counterpart in the
 * reference).  Same inputs, outputs and results as lg_policy_device on an
 * FP32 policy net, for callers that cannot call cudaMalloc at evaluation
 * time: a search thread in a process whose device memory is owned by
 * another allocator, a latency path that must not absorb cudaMalloc /
 * cudaFree's device-wide synchronisation, or a host callback where CUDA
 * allocation is not allowed.  Its scratch (activations, split-K partial
 * sums, logits when `logits` is NULL) is one static 8 MiB device array in
 * the library, held by every GPU that loads it until the process exits.
 *   - B is limited to 4 positions per call; larger B, or a net whose
 *     scratch would not fit, is rejected with LG_ERR_ARG and a message.
 *   - lg_create looks up the array's device address (cudaGetSymbolAddress)
 *     for its device when the context has an FP32 policy net, so calls
 *     only read that cached address.  (Were that lookup not done, the
 *     first call on a device would make it; such a first call should come
 *     before any stream capture.)
 *   - Every call, on every context, shares the one array: calls whose work
 *     overlaps on the GPU (different streams, or different host threads
 *     without ordering) race on it.  Nothing in it needs to start at zero.
 * All pointers are device memory; work is enqueued on `stream`. */
LG_API int lg_policy_device_static(lg_ctx *ctx, const uint8_t *planes, int B, float temperature,
                                   float *probs, float *logits, void *stream);

/* Autotuner.  For every power-of-two batch bucket up to max_batch, times the
 * context's nets with each kernel choice for the 3x3 layers of the
 * tensor-core nets (0: one launch per layer with 256-row tiles on the
 * transposed kernel, 1: one launch per layer with 128-row tiles, which put
 * twice as many CTAs on a small batch, 2: all 3x3 layers in one persistent
 * launch, 3: as 2 with the 5x5 first layer in the same launch),
 * for the first layer (0: 256-row, 1: 128-row tiles; unused by choices 3
 * and 4), and -- for buckets of at most 8 positions -- choice 4: every layer
 * of the net in one small-batch launch (FP32 nets: 0 = the generic per-layer
 * FP32 kernels, 4 = the small-batch kernel), and keeps the fastest.  With a
 * cache path, a table saved for the same device, SM count and net shapes is
 * loaded instead (unless force), and a new table is saved there (written to
 * a temporary file and renamed).  Without tuning (measured defaults): a
 * context with a 16-bit net uses choice 4 up to 2 positions and choice 3
 * above; an FP32-only context uses choice 4 up to 8 positions and its
 * per-layer kernels above.  No reference
 * counterpart (the OpenCL backend reads a fixed cfg_rowtiles,
 * OpenCL.cpp:634-646).  lg_tuning reports the choice for batch B; it returns
 * 1 once tuned, 0 if not, < 0 on error. */
LG_API int lg_autotune(lg_ctx *ctx, const char *cache_path, int force);
LG_API int lg_tuning(lg_ctx *ctx, int B, int *variant_3x3, int *variant_first);
/* Sets the kernel choice of B's bucket by hand (3x3: 0-4, first: 0-1); a
 * net that choice 4 does not cover runs its per-layer kernels. */
LG_API int lg_set_tuning(lg_ctx *ctx, int B, int variant_3x3, int variant_first);

/* ---------------------------------------------------------------------
 * Distilled student net (no reference counterpart; the reference trained
 * offline with Caffe, Network.cpp:1381-1509).  One trunk (5x5 c_in -> width,
 * n3x3 x 3x3 width -> width, ReLU) with a 1x1 policy head (softmax over
 * 361) and a 1x1 value head -> FC 361 -> fc_hidden (ReLU) -> FC -> tanh,
 * trained in FP32 on the GPU by this library's forward and backward kernels
 * with Adam.  Loss = KL(target policy || softmax) + value_weight *
 * (value - target)^2, averaged over the batch.
 *
 * Flat parameter layout (host side): per conv W[O][C][k][k] then b[O]; then
 * policy head w[width], b; value head w[width], b; W1[fc_hidden][361],
 * b1[fc_hidden], W2[fc_hidden], b2.  The trunk + policy head is a valid
 * lg_net_desc weight array for a policy net (head_k 1), and the trunk +
 * value head + FC one for a value net, so a trained student can be served
 * by lg_create at any precision.
 *
 * planes / targets are device pointers: planes [B][c_in][361] bytes, target
 * probabilities [B][361], target values [B] in [-1, 1]. */
typedef struct lg_student lg_student;
LG_API int lg_student_create(int device, int c_in, int width, int n3x3, int fc_hidden, int max_batch,
                             lg_student **out);
LG_API void lg_student_destroy(lg_student *st);
LG_API size_t lg_student_param_count(const lg_student *st);
LG_API int lg_student_set_params(lg_student *st, const float *host, size_t n);
LG_API int lg_student_get_params(lg_student *st, float *host, size_t n);
/* One Adam step (lr, betas 0.9 / 0.999, eps 1e-8); host_loss (optional)
 * receives {policy KL, value MSE} of the batch. */
LG_API int lg_student_train_step(lg_student *st, const uint8_t *planes, int B, const float *target_probs,
                                 const float *target_value, float lr, float value_weight, float *host_loss,
                                 void *stream);
/* Loss gradients in the flat host layout, no update (gradient checks). */
LG_API int lg_student_grads(lg_student *st, const uint8_t *planes, int B, const float *target_probs,
                            const float *target_value, float value_weight, float *host_grads,
                            float *host_loss);
/* FP32 forward: probabilities at temperature 1 and values (device). */
LG_API int lg_student_forward(lg_student *st, const uint8_t *planes, int B, float *probs, float *value,
                              void *stream);

/* The distilled student served for evaluation: BF16, one fused kernel for
 * the whole trunk (5x5 c_in -> 64, n3x3 x 3x3 64 -> 64, ReLU) and both 1x1
 * heads of two boards at a time, activations kept in shared memory; then the
 * softmax (with the policy's entropy) and the value FC.  Weights in the
 * lg_student flat layout with width 64 (lg_fast_param_count floats); c_in a
 * multiple of 4 up to 24.  No reference counterpart: the engine evaluates
 * every leaf with the full nets (UCTNode.cpp:74-121, Network.cpp:590-674).
 *
 * lg_fast_device is asynchronous on `stream` (device pointers; planes
 * 4-byte aligned, bytes 0 or 1 -- other values are read as their lowest
 * bit; logits and entropy may be NULL); lg_fast_status waits for the
 * stream and reports a kernel's error word (LG_ERR_DEVICE) if one gave up a
 * bounded wait. */
typedef struct lg_fast lg_fast;
LG_API size_t lg_fast_param_count(int c_in, int n3x3, int fc_hidden);
LG_API int lg_fast_create(int device, int c_in, int n3x3, int fc_hidden, int max_batch, const float *weights,
                          lg_fast **out);
LG_API int lg_fast_set_weights(lg_fast *f, const float *weights);
LG_API void lg_fast_destroy(lg_fast *f);
LG_API int lg_fast_device(lg_fast *f, const uint8_t *planes, int B, float temperature, float *probs,
                          float *logits, float *value, float *entropy, void *stream);
LG_API int lg_fast_status(lg_fast *f, void *stream);

/* The learned fast path for a batch of leaves: the student answers all B
 * positions; those whose policy entropy exceeds `threshold` nats are
 * compacted on the device, run through the full context's policy and value
 * nets (tensor-core nets on the persistent trunk kernel, batch size read on
 * the device) and written over the student's answers -- no host
 * synchronisation anywhere.  planes_p / planes_v: the positions' planes for
 * the full policy / value net ([B][c_in][361] each; the student reads
 * planes_p).  fallback (optional, [B] bytes): 1 where the full nets
 * answered; count (optional, one int): how many.  B <= the student's
 * max_batch.  Asynchronous on `stream`.  No reference counterpart (see
 * lg_fast). */
LG_API int lg_gated_device(lg_fast *student, lg_ctx *full, const uint8_t *planes_p, const uint8_t *planes_v,
                           int B, float temperature, float threshold, float *probs, float *value,
                           uint8_t *fallback, int32_t *count, void *stream);

/* Per-kernel timing for the roofline report.  lg_profile(ctx, 1) clears the
 * counters and brackets every kernel launched by later device-pointer calls
 * (lg_policy_device / lg_value_device) with CUDA events on the launching
 * stream; lg_profile_read waits for those events and returns, for one kernel
 * kind, the number of launches and their summed duration.  No reference
 * counterpart (the reference prints only wall-clock p/s, Network.cpp:147-199). */
#define LG_PROF_TC_3X3 0   /* tensor-core 3x3 trunk conv */
#define LG_PROF_TC_HEAD 1  /* tensor-core 3x3 conv with the fused 1x1 head */
#define LG_PROF_TC_FIRST 2 /* tensor-core 5x5 first layer */
#define LG_PROF_FP32_CONV 3 /* FP32 conv (+ split-K reduction) */
#define LG_PROF_OTHER 4    /* FP32 plane packing and head conv */
#define LG_PROF_TC_TRUNK 5 /* persistent kernel running all 3x3 layers (incl. the fused head) */
#define LG_PROF_PACK 6     /* tensor-core plane packing (planes -> expanded BF16 rows) */
#define LG_PROF_TAIL 7     /* softmax or value head (with the next chunk's packing in chained calls) */
#define LG_PROF_LAT 8      /* small-batch kernel: a whole net in one launch */
#define LG_PROF_KINDS 9
LG_API int lg_profile(lg_ctx *ctx, int enable);
LG_API int lg_profile_read(lg_ctx *ctx, int kind, long long *launches, double *total_ms);

/* Test hook (host-side fault injection): the n-th device call from now
 * (n >= 1) fails with LG_ERR_CUDA before it reaches the GPU; 0 disarms. */
LG_API int lg_inject_fault(lg_ctx *ctx, int nth_call);

/* Test hook (device-side bounded waits): the next launch of kernel `kind`
 * (0: the persistent trunk -- the first item of the second 3x3 layer; 1:
 * the small-batch kernel -- row 0 of the second layer) waits for a flag
 * that nothing publishes, with its wait limits cut to `polls` (0: 4096).
 * The wait runs out, the kernel records an error word and unwinds (no trap,
 * no fault), a blocking call returns LG_ERR_DEVICE, and the context keeps
 * working.  kind -1 disarms.  No reference counterpart (the engine's own
 * final wait, OpenCL.cpp:575-577, is unbounded). */
LG_API int lg_inject_stall(lg_ctx *ctx, int kind, int polls);

#ifdef __cplusplus
}
#endif
#endif

/*
 * leela_oracle.h -- CPU restatement of Leela's network evaluation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path
 * in leela_gb300: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  The product never calls it.
 *
 * What it restates (reference file:line):
 *   - convolve<k,C,O>    Network.cpp:345-393  im2col + sgemm + bias + ELU
 *   - im2col<C,k>        Im2Col.h:9-50        'same' zero padding on 19x19
 *   - innerproduct<I,O>  Network.cpp:395-423  sgemv + bias + ELU if O > 1
 *   - softmax            Network.cpp:450-469  max-subtracted, temperature
 *   - rotate_nn_idx      Network.cpp:1341-1379 (8 dihedral symmetries)
 *   - value mapping      Network.cpp:735-737  (1 + tanh(x)) / 2
 * generalised over the activation (ELU as in the reference, ReLU for the
 * benchmark nets), the head filter size (3x3 as in the reference, 1x1 for
 * the benchmark nets) and the value mapping (tanh or (1+tanh)/2).
 *
 * Two arithmetic widths: FP32 (same operation order per output as the
 * reference's im2col+GEMM: sum over c, ky, kx) and FP64 (every product and
 * sum in double; the "FP64 host oracle" for the BF16 / FP8 error figures).
 *
 * Parity pin: tests/golden holds outputs of the reference's own compiled
 * convolve<>/innerproduct<>/softmax code (built from the reference sources by
 * oracle/Makefile) on identical positions and weights; the tests check this
 * restatement against them.
 */
#ifndef LEELA_ORACLE_H
#define LEELA_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OR_BOARD 19
#define OR_POINTS 361

/* Net shape.  Conv layers, in order:
 *   conv 0      : 5x5, c_in   -> width1
 *   conv 1..n3x3: 3x3, width1 -> width, then width -> width
 *   head conv   : head_k x head_k, width -> 1
 * Activation `act` after every conv but the head; after the head conv only
 * if act_head.  Value nets (value_head = 1) add FC 361 -> fc_hidden (+act)
 * and FC fc_hidden -> 1, then the value map.
 *
 * Flat weight layout (the order weights are drawn and stored):
 *   for each conv: W[O][C][k][k] then b[O]
 *   value nets   : W1[fc_hidden][361], b1[fc_hidden], W2[fc_hidden], b2[1]
 */
typedef struct or_net {
    int c_in;
    int width1;
    int width;
    int n3x3;
    int head_k;
    int act;        /* 0 = ELU, 1 = ReLU */
    int act_head;   /* 1 = activation after the head conv too */
    int value_head; /* 0 = policy (361 logits), 1 = value (FC head) */
    int fc_hidden;
    int value_map;  /* 0 = tanh, 1 = (1 + tanh) / 2, 2 = none (the FC output itself) */
} or_net;

int or_n_conv(const or_net *n);
void or_conv_shape(const or_net *n, int layer, int *k, int *cin, int *cout);
size_t or_weight_count(const or_net *n);
size_t or_conv_weight_offset(const or_net *n, int layer); /* offset of W; b follows W */
size_t or_fc_weight_offset(const or_net *n);

/* He-normal N(0, 2/fan_in) weights, zero biases, drawn layer by layer from
 * one splitmix64 stream seeded with `seed`.  Uses only IEEE basic
 * operations and sqrt, so the values are bit-identical on every platform
 * (the library is compiled with -ffp-contract=off). */
void or_he_weights(const or_net *n, uint64_t seed, float *w);
double or_det_log(double x);
uint64_t or_checksum_f32(const float *x, size_t count);

/* Optional BLAS hooks (row-major cblas_sgemm / cblas_dgemm signature). When
 * set, the forward passes use them for the per-layer GEMM, as the
 * reference does; otherwise plain loops. */
typedef void (*or_sgemm_fn)(int order, int ta, int tb, int M, int N, int K, float alpha,
                            const float *A, int lda, const float *B, int ldb, float beta,
                            float *C, int ldc);
typedef void (*or_dgemm_fn)(int order, int ta, int tb, int M, int N, int K, double alpha,
                            const double *A, int lda, const double *B, int ldb, double beta,
                            double *C, int ldc);
void or_set_blas(or_sgemm_fn s, or_dgemm_fn d);

/* One position: planes [c_in][361] of 0/1 bytes, already rotated.
 * Policy nets write 361 pre-softmax logits to `out` (after the head
 * activation when act_head).  Value nets write the mapped value to out[0].
 * If `acts` is non-NULL it receives every conv layer's output, [361 * cout]
 * per layer, back to back.  Returns 0, or -1 on bad arguments. */
int or_forward_f32(const or_net *n, const float *w, const uint8_t *planes, float *out,
                   float *acts);
int or_forward_f64(const or_net *n, const float *w, const uint8_t *planes, double *out);

/* Batched helpers over B positions, [B][c_in][361] planes. nthreads <= 0:
 * one thread per online CPU.  Each position runs on one thread. */
int or_forward_batch_f32(const or_net *n, const float *w, const uint8_t *planes, int B,
                         float *out, int nthreads);
int or_forward_batch_f64(const or_net *n, const float *w, const uint8_t *planes, int B,
                         double *out, int nthreads);

void or_softmax_f32(const float *x, int count, float temperature, float *out);
void or_softmax_f64(const double *x, int count, double temperature, double *out);

int or_rotate_nn_idx(int vertex, int symmetry);
int or_rev_rotate_nn_idx(int vertex, int symmetry);
/* planes_out[c][i] = planes_in[c][rotate_nn_idx(i, sym)] (Network.cpp:765-773). */
void or_rotate_planes(const uint8_t *in, int channels, int symmetry, uint8_t *out);

/* E4M3 quantisation as the FP8 weight variant defines it: per output channel
 * scale = max|w| / 448, q = round-to-nearest-even(w / scale) in E4M3
 * (saturating at +-448).  Writes the dequantised weights q * scale. */
float or_e4m3_round(float x);
void or_fp8_dequant_conv(const float *w, int cout, int per_out, float *wq, float *scales);
float or_bf16_round(float x);

/* Timed CPU baseline: `iters` forward passes of the policy and the value net
 * over the given positions, one position per thread on `nthreads` threads.
 * Returns elapsed seconds. */
double or_time_pair_f32(const or_net *pol, const float *wp, const or_net *val, const float *wv,
                        const uint8_t *planes_p, const uint8_t *planes_v, int npos, int iters,
                        int nthreads);

/* Input planes 0..nplanes-1 (nplanes <= 32) of the policy (which = 0) or
 * value (which = 1) set, restating Network::gather_features_policy /
 * gather_features_value (Network.cpp:883-1046, 1048-1201): colours, string
 * liberties (FastBoard::count_rliberties, FastBoard.cpp:2482-2508),
 * after-move liberties of both colours (FastBoard::after_liberties,
 * FastBoard.cpp:2511-2528; 0 for a suicide), the ladder reader's planes
 * (FastBoard::saving_size / check_losing_ladder / check_winning_ladder,
 * FastBoard.cpp:1273-1292, 2530-2837), ko point, last two moves, komi and
 * third line.  squares[361]: 0 black, 1 white, 2 empty, point y*19+x;
 * moves[4] (may be NULL when nplanes <= 24): last move, the move before it,
 * ko point (point index, -1 none), white-has-komi flag; planes[nplanes][361]. */
void or_gather_planes(const int8_t *squares, int to_move, const int32_t *moves, int which, int nplanes,
                      uint8_t *planes);

/* A board reached by k uniformly random legal moves from the empty board
 * (captures applied, suicide excluded, simple ko ignored), for parity cases
 * beyond the fixture positions.  Writes squares[361]; returns the side to
 * move (0 black, 1 white). */
int or_random_board(uint64_t seed, int k, int8_t *squares);

/* A position as the benchmark configurations define them: from the empty
 * board, k ~ U[0, kmax] uniform legal non-pass moves (simple ko, no
 * suicide), from a splitmix64 stream seeded with `seed`.  Writes
 * squares[361] and moves[4] (last move, the move before it, ko point,
 * white-has-komi flag); returns the side to move. */
int or_config_board(uint64_t seed, int kmax, int8_t *squares, int32_t *moves);
void or_config_boards(uint64_t base, int start, int n, int kmax, int8_t *squares, int32_t *moves,
                      int8_t *to_move);

#ifdef __cplusplus
}
#endif
#endif

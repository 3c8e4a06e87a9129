/*
 * leela_oracle.c -- CPU restatement of Leela's network evaluation path.
 *
 * TEST INFRASTRUCTURE ONLY (see leela_oracle.h).  Compiled with
 * -ffp-contract=off so that no multiply-add is fused and the FP32 and FP64
 * results, and the weight generator, are the same on x86 and Arm hosts.
 */
#define _GNU_SOURCE
#include "leela_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

/* ------------------------------------------------------------------ shape */

int or_n_conv(const or_net *n) { return 1 + n->n3x3 + 1; }

void or_conv_shape(const or_net *n, int layer, int *k, int *cin, int *cout) {
    int nc = or_n_conv(n);
    if (layer == 0) {
        *k = 5; *cin = n->c_in; *cout = n->width1;
    } else if (layer < nc - 1) {
        *k = 3; *cin = (layer == 1) ? n->width1 : n->width; *cout = n->width;
    } else {
        *k = n->head_k; *cin = (n->n3x3 > 0) ? n->width : n->width1; *cout = 1;
    }
}

static size_t conv_params(const or_net *n, int layer) {
    int k, ci, co;
    or_conv_shape(n, layer, &k, &ci, &co);
    return (size_t)co * ci * k * k + (size_t)co;
}

size_t or_conv_weight_offset(const or_net *n, int layer) {
    size_t off = 0;
    for (int l = 0; l < layer; ++l) off += conv_params(n, l);
    return off;
}

size_t or_fc_weight_offset(const or_net *n) { return or_conv_weight_offset(n, or_n_conv(n)); }

size_t or_weight_count(const or_net *n) {
    size_t c = or_fc_weight_offset(n);
    if (n->value_head) c += (size_t)n->fc_hidden * OR_POINTS + n->fc_hidden + n->fc_hidden + 1;
    return c;
}

/* ---------------------------------------------------- deterministic weights */

static uint64_t splitmix64(uint64_t *s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static double uniform_open(uint64_t *s) {
    /* (0,1): 53 random bits, offset by half an ulp of the grid. */
    return ((double)(splitmix64(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

/* Natural log from frexp and the atanh series ln(m) = 2 atanh((m-1)/(m+1)),
 * m in [0.5, 1): |t| <= 1/3, 30 terms reach well below double rounding. */
double or_det_log(double x) {
    int e;
    double m = frexp(x, &e);
    double t = (m - 1.0) / (m + 1.0);
    double t2 = t * t;
    double term = t;
    double sum = 0.0;
    for (int i = 0; i < 30; ++i) {
        sum = sum + term / (double)(2 * i + 1);
        term = term * t2;
    }
    return 2.0 * sum + (double)e * 0.69314718055994530942;
}

static double normal(uint64_t *s) {
    /* Marsaglia polar method, first variate of each accepted pair. */
    for (;;) {
        double u = 2.0 * uniform_open(s) - 1.0;
        double v = 2.0 * uniform_open(s) - 1.0;
        double q = u * u + v * v;
        if (q >= 1.0 || q == 0.0) continue;
        return u * sqrt(-2.0 * or_det_log(q) / q);
    }
}

static void fill_he(uint64_t *s, float *w, size_t count, int fan_in) {
    double sd = sqrt(2.0 / (double)fan_in);
    for (size_t i = 0; i < count; ++i) w[i] = (float)(normal(s) * sd);
}

void or_he_weights(const or_net *n, uint64_t seed, float *w) {
    uint64_t s = seed;
    int nc = or_n_conv(n);
    for (int l = 0; l < nc; ++l) {
        int k, ci, co;
        or_conv_shape(n, l, &k, &ci, &co);
        float *W = w + or_conv_weight_offset(n, l);
        size_t nw = (size_t)co * ci * k * k;
        fill_he(&s, W, nw, ci * k * k);
        memset(W + nw, 0, sizeof(float) * co);
    }
    if (n->value_head) {
        float *p = w + or_fc_weight_offset(n);
        fill_he(&s, p, (size_t)n->fc_hidden * OR_POINTS, OR_POINTS);
        p += (size_t)n->fc_hidden * OR_POINTS;
        memset(p, 0, sizeof(float) * n->fc_hidden);
        p += n->fc_hidden;
        fill_he(&s, p, (size_t)n->fc_hidden, n->fc_hidden);
        p += n->fc_hidden;
        p[0] = 0.0f;
    }
}

uint64_t or_checksum_f32(const float *x, size_t count) {
    /* FNV-1a over the raw bit patterns. */
    uint64_t h = 1469598103934665603ULL;
    const unsigned char *b = (const unsigned char *)x;
    for (size_t i = 0; i < count * sizeof(float); ++i) {
        h ^= b[i];
        h *= 1099511628211ULL;
    }
    return h;
}

/* ------------------------------------------------------------------ BLAS */

static or_sgemm_fn g_sgemm = NULL;
static or_dgemm_fn g_dgemm = NULL;
void or_set_blas(or_sgemm_fn s, or_dgemm_fn d) {
    g_sgemm = s;
    g_dgemm = d;
}
enum { ROW_MAJOR = 101, NO_TRANS = 111 };

/* ---------------------------------------------------------------- im2col */

/* 'same' zero padding on 19x19 (Im2Col.h:9-50): row (c, ky, kx), column p. */
#define DEFINE_IM2COL(NAME, T)                                                         \
    static void NAME(const T *in, int channels, int k, T *col) {                      \
        int pad = k / 2;                                                               \
        for (int c = 0; c < channels; ++c)                                             \
            for (int ky = 0; ky < k; ++ky)                                             \
                for (int kx = 0; kx < k; ++kx) {                                       \
                    T *dst = col + ((size_t)(c * k + ky) * k + kx) * OR_POINTS;        \
                    for (int y = 0; y < OR_BOARD; ++y) {                               \
                        int iy = y + ky - pad;                                         \
                        for (int x = 0; x < OR_BOARD; ++x) {                           \
                            int ix = x + kx - pad;                                     \
                            dst[y * OR_BOARD + x] =                                    \
                                (iy >= 0 && iy < OR_BOARD && ix >= 0 && ix < OR_BOARD) \
                                    ? in[(size_t)c * OR_POINTS + iy * OR_BOARD + ix]   \
                                    : (T)0;                                            \
                        }                                                              \
                    }                                                                  \
                }                                                                      \
    }
DEFINE_IM2COL(im2col_f32, float)
DEFINE_IM2COL(im2col_f64, double)

/* out[o][p] = sum_k W[o][k] col[k][p], accumulated in k order. */
static void gemm_f32(const float *W, const float *col, int O, int K, float *out) {
    if (g_sgemm) {
        g_sgemm(ROW_MAJOR, NO_TRANS, NO_TRANS, O, OR_POINTS, K, 1.0f, W, K, col, OR_POINTS, 0.0f,
                out, OR_POINTS);
        return;
    }
    for (int o = 0; o < O; ++o) {
        float *dst = out + (size_t)o * OR_POINTS;
        for (int p = 0; p < OR_POINTS; ++p) dst[p] = 0.0f;
        for (int kk = 0; kk < K; ++kk) {
            float wv = W[(size_t)o * K + kk];
            const float *src = col + (size_t)kk * OR_POINTS;
            for (int p = 0; p < OR_POINTS; ++p) dst[p] = dst[p] + wv * src[p];
        }
    }
}

static void gemm_f64(const double *W, const double *col, int O, int K, double *out) {
    if (g_dgemm) {
        g_dgemm(ROW_MAJOR, NO_TRANS, NO_TRANS, O, OR_POINTS, K, 1.0, W, K, col, OR_POINTS, 0.0,
                out, OR_POINTS);
        return;
    }
    for (int o = 0; o < O; ++o) {
        double *dst = out + (size_t)o * OR_POINTS;
        for (int p = 0; p < OR_POINTS; ++p) dst[p] = 0.0;
        for (int kk = 0; kk < K; ++kk) {
            double wv = W[(size_t)o * K + kk];
            const double *src = col + (size_t)kk * OR_POINTS;
            for (int p = 0; p < OR_POINTS; ++p) dst[p] = dst[p] + wv * src[p];
        }
    }
}

/* ----------------------------------------------------------- activations */

static float act_f32(float v, int act) {
    if (act == 0) return (v > 0.0f) ? v : (expf(v) - 1.0f); /* Network.cpp:382-383 */
    return (v > 0.0f) ? v : 0.0f;
}
static double act_f64(double v, int act) {
    if (act == 0) return (v > 0.0) ? v : (exp(v) - 1.0);
    return (v > 0.0) ? v : 0.0;
}

/* ------------------------------------------------------------- forward */

static int max_channels(const or_net *n) {
    int m = n->c_in;
    if (n->width1 > m) m = n->width1;
    if (n->width > m) m = n->width;
    return m;
}

static int valid_net(const or_net *n) {
    return n && n->c_in > 0 && n->width1 > 0 && n->width > 0 && n->n3x3 >= 0 &&
           (n->head_k == 1 || n->head_k == 3) && (n->act == 0 || n->act == 1) &&
           (!n->value_head || n->fc_hidden > 0);
}

int or_forward_f32(const or_net *n, const float *w, const uint8_t *planes, float *out,
                   float *acts) {
    if (!valid_net(n) || !w || !planes || !out) return -1;
    int mc = max_channels(n);
    float *a = malloc(sizeof(float) * mc * OR_POINTS);
    float *b = malloc(sizeof(float) * mc * OR_POINTS);
    float *col = malloc(sizeof(float) * (size_t)mc * 25 * OR_POINTS);
    if (!a || !b || !col) {
        free(a); free(b); free(col);
        return -1;
    }
    for (int i = 0; i < n->c_in * OR_POINTS; ++i) a[i] = (float)planes[i];
    int nc = or_n_conv(n);
    for (int l = 0; l < nc; ++l) {
        int k, ci, co;
        or_conv_shape(n, l, &k, &ci, &co);
        const float *W = w + or_conv_weight_offset(n, l);
        const float *bias = W + (size_t)co * ci * k * k;
        im2col_f32(a, ci, k, col);
        gemm_f32(W, col, co, ci * k * k, b);
        int do_act = (l < nc - 1) || n->act_head;
        for (int o = 0; o < co; ++o)
            for (int p = 0; p < OR_POINTS; ++p) {
                float v = bias[o] + b[(size_t)o * OR_POINTS + p];
                b[(size_t)o * OR_POINTS + p] = do_act ? act_f32(v, n->act) : v;
            }
        if (acts) {
            memcpy(acts, b, sizeof(float) * co * OR_POINTS);
            acts += (size_t)co * OR_POINTS;
        }
        float *t = a; a = b; b = t;
    }
    if (!n->value_head) {
        memcpy(out, a, sizeof(float) * OR_POINTS);
    } else {
        /* innerproduct<361, H> then innerproduct<H, 1> (Network.cpp:395-423). */
        const float *W1 = w + or_fc_weight_offset(n);
        const float *b1 = W1 + (size_t)n->fc_hidden * OR_POINTS;
        const float *W2 = b1 + n->fc_hidden;
        const float *b2 = W2 + n->fc_hidden;
        for (int o = 0; o < n->fc_hidden; ++o) {
            float s = 0.0f;
            for (int i = 0; i < OR_POINTS; ++i) s = s + W1[(size_t)o * OR_POINTS + i] * a[i];
            b[o] = act_f32(b1[o] + s, n->act);
        }
        float s = 0.0f;
        for (int i = 0; i < n->fc_hidden; ++i) s = s + W2[i] * b[i];
        float x = b2[0] + s;
        out[0] = n->value_map == 2 ? x : (n->value_map ? (1.0f + tanhf(x)) / 2.0f : tanhf(x));
    }
    free(a); free(b); free(col);
    return 0;
}

int or_forward_f64(const or_net *n, const float *w, const uint8_t *planes, double *out) {
    if (!valid_net(n) || !w || !planes || !out) return -1;
    int mc = max_channels(n);
    double *a = malloc(sizeof(double) * mc * OR_POINTS);
    double *b = malloc(sizeof(double) * mc * OR_POINTS);
    double *col = malloc(sizeof(double) * (size_t)mc * 25 * OR_POINTS);
    double *Wd = malloc(sizeof(double) * (size_t)mc * mc * 25);
    if (!a || !b || !col || !Wd) {
        free(a); free(b); free(col); free(Wd);
        return -1;
    }
    for (int i = 0; i < n->c_in * OR_POINTS; ++i) a[i] = (double)planes[i];
    int nc = or_n_conv(n);
    for (int l = 0; l < nc; ++l) {
        int k, ci, co;
        or_conv_shape(n, l, &k, &ci, &co);
        const float *W = w + or_conv_weight_offset(n, l);
        size_t nw = (size_t)co * ci * k * k;
        for (size_t i = 0; i < nw; ++i) Wd[i] = (double)W[i];
        const float *bias = W + nw;
        im2col_f64(a, ci, k, col);
        gemm_f64(Wd, col, co, ci * k * k, b);
        int do_act = (l < nc - 1) || n->act_head;
        for (int o = 0; o < co; ++o)
            for (int p = 0; p < OR_POINTS; ++p) {
                double v = (double)bias[o] + b[(size_t)o * OR_POINTS + p];
                b[(size_t)o * OR_POINTS + p] = do_act ? act_f64(v, n->act) : v;
            }
        double *t = a; a = b; b = t;
    }
    if (!n->value_head) {
        memcpy(out, a, sizeof(double) * OR_POINTS);
    } else {
        const float *W1 = w + or_fc_weight_offset(n);
        const float *b1 = W1 + (size_t)n->fc_hidden * OR_POINTS;
        const float *W2 = b1 + n->fc_hidden;
        const float *b2 = W2 + n->fc_hidden;
        for (int o = 0; o < n->fc_hidden; ++o) {
            double s = 0.0;
            for (int i = 0; i < OR_POINTS; ++i) s += (double)W1[(size_t)o * OR_POINTS + i] * a[i];
            b[o] = act_f64((double)b1[o] + s, n->act);
        }
        double s = 0.0;
        for (int i = 0; i < n->fc_hidden; ++i) s += (double)W2[i] * b[i];
        double x = (double)b2[0] + s;
        out[0] = n->value_map == 2 ? x : (n->value_map ? (1.0 + tanh(x)) / 2.0 : tanh(x));
    }
    free(a); free(b); free(col); free(Wd);
    return 0;
}

/* -------------------------------------------------------------- threads */

typedef struct {
    const or_net *n;
    const float *w;
    const uint8_t *planes;
    void *out;
    int begin, end, f64, rc;
} batch_job;

static void *batch_worker(void *arg) {
    batch_job *j = (batch_job *)arg;
    int per_in = j->n->c_in * OR_POINTS;
    int per_out = j->n->value_head ? 1 : OR_POINTS;
    for (int i = j->begin; i < j->end && j->rc == 0; ++i) {
        if (j->f64)
            j->rc = or_forward_f64(j->n, j->w, j->planes + (size_t)i * per_in,
                                   (double *)j->out + (size_t)i * per_out);
        else
            j->rc = or_forward_f32(j->n, j->w, j->planes + (size_t)i * per_in,
                                   (float *)j->out + (size_t)i * per_out, NULL);
    }
    return NULL;
}

static int resolve_threads(int nthreads, int B) {
    if (nthreads <= 0) nthreads = (int)sysconf(_SC_NPROCESSORS_ONLN);
    if (nthreads < 1) nthreads = 1;
    if (nthreads > B) nthreads = B;
    if (nthreads > 256) nthreads = 256;
    return nthreads;
}

static int run_batch(const or_net *n, const float *w, const uint8_t *planes, int B, void *out,
                     int nthreads, int f64) {
    if (B <= 0) return 0;
    nthreads = resolve_threads(nthreads, B);
    pthread_t tid[256];
    batch_job jobs[256];
    for (int t = 0; t < nthreads; ++t) {
        jobs[t] = (batch_job){n, w, planes, out, (int)((long)B * t / nthreads),
                              (int)((long)B * (t + 1) / nthreads), f64, 0};
        pthread_create(&tid[t], NULL, batch_worker, &jobs[t]);
    }
    int rc = 0;
    for (int t = 0; t < nthreads; ++t) {
        pthread_join(tid[t], NULL);
        if (jobs[t].rc) rc = jobs[t].rc;
    }
    return rc;
}

int or_forward_batch_f32(const or_net *n, const float *w, const uint8_t *planes, int B,
                         float *out, int nthreads) {
    return run_batch(n, w, planes, B, out, nthreads, 0);
}
int or_forward_batch_f64(const or_net *n, const float *w, const uint8_t *planes, int B,
                         double *out, int nthreads) {
    return run_batch(n, w, planes, B, out, nthreads, 1);
}

/* -------------------------------------------------------------- softmax */

/* Network.cpp:450-469: alpha = max/T; p_i = exp(x_i/T - alpha) / sum. */
void or_softmax_f32(const float *x, int count, float temperature, float *out) {
    float alpha = x[0];
    for (int i = 1; i < count; ++i)
        if (x[i] > alpha) alpha = x[i];
    alpha /= temperature;
    float denom = 0.0f;
    for (int i = 0; i < count; ++i) {
        float v = expf((x[i] / temperature) - alpha);
        out[i] = v;
        denom += v;
    }
    for (int i = 0; i < count; ++i) out[i] = out[i] / denom;
}

void or_softmax_f64(const double *x, int count, double temperature, double *out) {
    double alpha = x[0];
    for (int i = 1; i < count; ++i)
        if (x[i] > alpha) alpha = x[i];
    alpha /= temperature;
    double denom = 0.0;
    for (int i = 0; i < count; ++i) {
        double v = exp((x[i] / temperature) - alpha);
        out[i] = v;
        denom += v;
    }
    for (int i = 0; i < count; ++i) out[i] = out[i] / denom;
}

/* ------------------------------------------------------------- symmetry */

/* Network.cpp:1360-1379: symmetries 4..7 transpose first, then 0..3 are
 * identity, flip y, flip x, flip both. */
int or_rotate_nn_idx(int vertex, int symmetry) {
    int x = vertex % OR_BOARD, y = vertex / OR_BOARD;
    if (symmetry >= 4) {
        int t = x; x = y; y = t;
        symmetry -= 4;
    }
    int nx = (symmetry & 2) ? OR_BOARD - 1 - x : x;
    int ny = (symmetry & 1) ? OR_BOARD - 1 - y : y;
    return ny * OR_BOARD + nx;
}

/* Network.cpp:1341-1346: the inverse of 5 is 6 and of 6 is 5. */
int or_rev_rotate_nn_idx(int vertex, int symmetry) {
    static const int invert[8] = {0, 1, 2, 3, 4, 6, 5, 7};
    return or_rotate_nn_idx(vertex, invert[symmetry]);
}

void or_rotate_planes(const uint8_t *in, int channels, int symmetry, uint8_t *out) {
    for (int c = 0; c < channels; ++c)
        for (int i = 0; i < OR_POINTS; ++i)
            out[c * OR_POINTS + i] = in[c * OR_POINTS + or_rotate_nn_idx(i, symmetry)];
}

/* ------------------------------------------------------------ low precision */

/* Round-to-nearest-even onto E4M3 (bias 7, 3 mantissa bits, max 448, no
 * infinities), by scaling to the binade's integer grid. */
float or_e4m3_round(float x) {
    if (x != x) return x;
    float a = fabsf(x);
    if (a >= 448.0f) return x < 0 ? -448.0f : 448.0f;
    if (a == 0.0f) return x;
    int e;
    frexpf(a, &e);          /* a = m * 2^e, m in [0.5, 1) -> unbiased exponent e-1 */
    int ex = e - 1;
    if (ex < -6) ex = -6;   /* subnormal range: step 2^-9 */
    float step = ldexpf(1.0f, ex - 3);
    float q = rintf(a / step) * step; /* rintf: ties to even in the default mode */
    if (q > 448.0f) q = 448.0f;
    return x < 0 ? -q : q;
}

void or_fp8_dequant_conv(const float *w, int cout, int per_out, float *wq, float *scales) {
    for (int o = 0; o < cout; ++o) {
        float m = 0.0f;
        for (int i = 0; i < per_out; ++i) {
            float a = fabsf(w[(size_t)o * per_out + i]);
            if (a > m) m = a;
        }
        float s = (m > 0.0f) ? m / 448.0f : 1.0f;
        scales[o] = s;
        for (int i = 0; i < per_out; ++i)
            wq[(size_t)o * per_out + i] = or_e4m3_round(w[(size_t)o * per_out + i] / s) * s;
    }
}

float or_bf16_round(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return x;
    u = (u + 0x7fffu + ((u >> 16) & 1u)) & 0xffff0000u;
    float r;
    memcpy(&r, &u, 4);
    return r;
}

/* ------------------------------------------------------------- timing */

typedef struct {
    const or_net *pol, *val;
    const float *wp, *wv;
    const uint8_t *pp, *pv;
    int npos, iters, tid, nthreads;
} pair_job;

static void *pair_worker(void *arg) {
    pair_job *j = (pair_job *)arg;
    float out[OR_POINTS];
    int per_p = j->pol->c_in * OR_POINTS, per_v = j->val->c_in * OR_POINTS;
    for (int it = j->tid; it < j->iters; it += j->nthreads) {
        int i = it % j->npos;
        or_forward_f32(j->pol, j->wp, j->pp + (size_t)i * per_p, out, NULL);
        or_forward_f32(j->val, j->wv, j->pv + (size_t)i * per_v, out, NULL);
    }
    return NULL;
}

double or_time_pair_f32(const or_net *pol, const float *wp, const or_net *val, const float *wv,
                        const uint8_t *planes_p, const uint8_t *planes_v, int npos, int iters,
                        int nthreads) {
    nthreads = resolve_threads(nthreads, iters);
    pthread_t tid[256];
    pair_job jobs[256];
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int t = 0; t < nthreads; ++t) {
        jobs[t] = (pair_job){pol, val, wp, wv, planes_p, planes_v, npos, iters, t, nthreads};
        pthread_create(&tid[t], NULL, pair_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(tid[t], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

/* ------------------------------------------------------- input planes */

#define GB_EMPTY 2

static int gb_nbrs(int p, int *out) {
    int x = p % 19, y = p / 19, n = 0;
    if (x > 0) out[n++] = p - 1;
    if (x < 18) out[n++] = p + 1;
    if (y > 0) out[n++] = p - 19;
    if (y < 18) out[n++] = p + 19;
    return n;
}

/* Flood-fills the string through p; marks its stones in `in` (1) and
 * returns its liberty count.  Stones go to list[] when it is given. */
static int gb_string(const int8_t *sq, int p, uint8_t *in, int *list, int *nlist) {
    int stack[OR_POINTS], sp = 0, n = 0, libs = 0;
    uint8_t seen_lib[OR_POINTS];
    memset(seen_lib, 0, sizeof seen_lib);
    int8_t c = sq[p];
    in[p] = 1;
    stack[sp++] = p;
    while (sp) {
        int q = stack[--sp], nb[4];
        if (list) list[n++] = q;
        int m = gb_nbrs(q, nb);
        for (int k = 0; k < m; ++k) {
            int r = nb[k];
            if (sq[r] == GB_EMPTY) {
                if (!seen_lib[r]) { seen_lib[r] = 1; ++libs; }
            } else if (sq[r] == c && !in[r]) {
                in[r] = 1;
                stack[sp++] = r;
            }
        }
    }
    if (nlist) *nlist = n;
    return libs;
}

static int gb_libs(const int8_t *sq, int p) {
    uint8_t in[OR_POINTS];
    memset(in, 0, sizeof in);
    return gb_string(sq, p, in, NULL, NULL);
}

/* Plays `color` at the empty point p on a copy of the board: removes the
 * opponent strings left without liberties, then returns the liberties of
 * the string through p, or 0 when that string has none (a suicide). */
static int gb_after(const int8_t *sq, int color, int p) {
    int8_t b[OR_POINTS];
    memcpy(b, sq, sizeof b);
    b[p] = (int8_t)color;
    int nb[4], m = gb_nbrs(p, nb);
    for (int k = 0; k < m; ++k) {
        int r = nb[k];
        if (b[r] == 1 - color && gb_libs(b, r) == 0) {
            uint8_t in[OR_POINTS];
            int list[OR_POINTS], n;
            memset(in, 0, sizeof in);
            gb_string(b, r, in, list, &n);
            for (int i = 0; i < n; ++i) b[list[i]] = GB_EMPTY;
        }
    }
    return gb_libs(b, p);
}

/* ---- ladder reader (FastBoard.cpp:1273-1292, 1342-1470, 2429-2442,
 * 2530-2564, 2647-2837), on a plain board: string liberties are exact
 * counts, as the reference's incrementally kept m_libs are. */

static int gb_count_empty(const int8_t *b, int v) {
    int nb[4], m = gb_nbrs(v, nb), n = 0;
    for (int k = 0; k < m; ++k) n += b[nb[k]] == GB_EMPTY;
    return n;
}

static int gb_size(const int8_t *b, int q) {
    uint8_t in[OR_POINTS];
    int list[OR_POINTS], n;
    memset(in, 0, sizeof in);
    gb_string(b, q, in, list, &n);
    return n;
}

/* Up to `want` distinct liberties of the string through q, into out[];
 * returns how many were found. */
static int gb_liberties(const int8_t *b, int q, int want, int *out) {
    uint8_t in[OR_POINTS];
    int list[OR_POINTS], n, cnt = 0;
    memset(in, 0, sizeof in);
    gb_string(b, q, in, list, &n);
    for (int i = 0; i < n && cnt < want; ++i) {
        int nb[4], m = gb_nbrs(list[i], nb);
        for (int k = 0; k < m && cnt < want; ++k) {
            int r = nb[k], dup = 0;
            if (b[r] != GB_EMPTY) continue;
            for (int j = 0; j < cnt; ++j) dup |= out[j] == r;
            if (!dup) out[cnt++] = r;
        }
    }
    return cnt;
}

static void gb_remove_string(int8_t *b, int q) {
    uint8_t in[OR_POINTS];
    int list[OR_POINTS], n;
    memset(in, 0, sizeof in);
    gb_string(b, q, in, list, &n);
    for (int i = 0; i < n; ++i) b[list[i]] = GB_EMPTY;
}

/* FastBoard::update_board_fast: place, capture opponent strings left without
 * liberties, remove the new string if it has none. */
static void gb_play(int8_t *b, int color, int v) {
    int nb[4], m = gb_nbrs(v, nb);
    b[v] = (int8_t)color;
    for (int k = 0; k < m; ++k)
        if (b[nb[k]] == 1 - color && gb_libs(b, nb[k]) == 0) gb_remove_string(b, nb[k]);
    if (gb_libs(b, v) == 0) gb_remove_string(b, v);
}

/* FastBoard::minimum_elib_count: fewest liberties among the opponent strings
 * next to the point v itself (100 if none). */
static int gb_min_elib(const int8_t *b, int color, int v) {
    int nb[4], m = gb_nbrs(v, nb), best = 100;
    for (int k = 0; k < m; ++k)
        if (b[nb[k]] == 1 - color) {
            int l = gb_libs(b, nb[k]);
            if (l < best) best = l;
        }
    return best;
}

/* FastBoard::is_suicide: no empty neighbour, every own neighbour string in
 * atari (its liberty is v), no opponent neighbour string in atari. */
static int gb_is_suicide(const int8_t *b, int v, int color) {
    if (gb_count_empty(b, v) > 0) return 0;
    int nb[4], m = gb_nbrs(v, nb);
    for (int k = 0; k < m; ++k) {
        int l = gb_libs(b, nb[k]);
        if (b[nb[k]] == color ? l > 1 : l <= 1) return 0;
    }
    return 1;
}

/* FastBoard::self_atari: fewer than two empty neighbours, no capture and no
 * connection to a string of 3+ liberties, and v, the empty neighbours and
 * the liberties of the own neighbour strings (those with 2+ liberties)
 * number at most two. */
static int gb_self_atari(const int8_t *b, int color, int v) {
    if (gb_count_empty(b, v) >= 2) return 0;
    int nb[4], m = gb_nbrs(v, nb);
    for (int k = 0; k < m; ++k) {
        int c = b[nb[k]];
        if (c == GB_EMPTY) continue;
        int l = gb_libs(b, nb[k]);
        if ((c == 1 - color && l <= 1) || (c == color && l >= 3)) return 0;
    }
    int set[8], cnt = 0;
    set[cnt++] = v;
    for (int k = 0; k < m; ++k) {
        int r = nb[k];
        if (b[r] == GB_EMPTY) {
            int dup = 0;
            for (int j = 0; j < cnt; ++j) dup |= set[j] == r;
            if (!dup) set[cnt++] = r;
        } else if (b[r] == color && gb_libs(b, r) > 1) {
            int libs[4], nl = gb_liberties(b, r, 4, libs);
            for (int i = 0; i < nl; ++i) {
                int dup = 0;
                for (int j = 0; j < cnt; ++j) dup |= set[j] == libs[i];
                if (!dup && cnt < 8) set[cnt++] = libs[i];
            }
        }
        if (cnt > 2) return 0;
    }
    return 1;
}

/* FastBoard::saving_size: the size of an own neighbour string in atari whose
 * saving move (its liberty) is not a self-atari, else 0. */
static int gb_saving_size(const int8_t *b, int color, int v) {
    int nb[4], m = gb_nbrs(v, nb);
    for (int k = 0; k < m; ++k) {
        if (b[nb[k]] != color || gb_libs(b, nb[k]) > 1) continue;
        int lib;
        if (gb_liberties(b, nb[k], 1, &lib) == 1 && !gb_self_atari(b, color, lib)) return gb_size(b, nb[k]);
    }
    return 0;
}

/* FastBoard::check_losing_ladder: `color` (to move) saves the string in
 * atari next to vtx by playing there; true when the attacker can keep it in
 * atari until it dies. */
static int gb_losing_ladder(const int8_t *board, int color, int vtx, int branching) {
    if (branching > 5) return 0;
    int elib = gb_min_elib(board, color, vtx);
    if (elib == 0 || elib == 1) return 0;
    /* the own strings in atari next to vtx: exactly one, and it cannot
     * capture an attacker */
    int nb[4], m = gb_nbrs(vtx, nb), crit = -1, ncrit = 0;
    uint8_t in_crit[OR_POINTS];
    memset(in_crit, 0, sizeof in_crit);
    for (int k = 0; k < m; ++k) {
        int r = nb[k];
        if (board[r] != color || gb_libs(board, r) > 1) continue;
        if (!in_crit[r]) {
            int list[OR_POINTS], n;
            gb_string(board, r, in_crit, list, &n);
            ++ncrit;
            crit = r;
        }
    }
    if (ncrit != 1) return 0;
    {
        uint8_t in[OR_POINTS];
        int list[OR_POINTS], n;
        memset(in, 0, sizeof in);
        gb_string(board, crit, in, list, &n);
        for (int i = 0; i < n; ++i) {
            int nb2[4], m2 = gb_nbrs(list[i], nb2);
            for (int k = 0; k < m2; ++k)
                if (board[nb2[k]] == 1 - color && gb_libs(board, nb2[k]) <= 1) return 0;
        }
    }
    int8_t b[OR_POINTS];
    memcpy(b, board, sizeof b);
    int atari = vtx;
    gb_play(b, color, vtx);
    for (;;) {
        if (b[atari] == GB_EMPTY) return 1;           /* the escape was a suicide */
        int nl = gb_libs(b, atari);
        if (nl == 1) return 1;                          /* self-atari */
        if (nl >= 3) return 0;                          /* escaped */
        if (gb_min_elib(b, color, atari) == 1) return 0; /* counter-atari */
        int lib[2];
        gb_liberties(b, atari, 2, lib);
        if (gb_count_empty(b, lib[0]) == 3 && gb_count_empty(b, lib[1]) == 3) return 0;
        int l0 = gb_after(b, color, lib[0]), l1 = gb_after(b, color, lib[1]);
        int s0 = gb_is_suicide(b, lib[0], 1 - color) || gb_self_atari(b, 1 - color, lib[0]);
        int s1 = gb_is_suicide(b, lib[1], 1 - color) || gb_self_atari(b, 1 - color, lib[1]);
        if (s0 && s1) return 0;
        if (s0) l1 = l0 + 1;
        if (s1) l0 = l1 + 1;
        if (l0 == l1) {
            int8_t b2[OR_POINTS];
            memcpy(b2, b, sizeof b2);
            gb_play(b2, 1 - color, lib[0]);
            int r1 = gb_losing_ladder(b2, color, lib[1], branching + 1);
            memcpy(b2, b, sizeof b2);
            gb_play(b2, 1 - color, lib[1]);
            int r2 = gb_losing_ladder(b2, color, lib[0], branching + 1);
            return r1 || r2;
        }
        gb_play(b, 1 - color, l0 > l1 ? lib[0] : lib[1]);
        /* the attacker's stone stands (neither suicide nor self-atari was
         * chosen) and captures no stone next to the saved string, so the
         * string has exactly one liberty: the next saving move */
        int next;
        if (gb_liberties(b, atari, 2, lib) != 1) return 0;
        next = lib[0];
        gb_play(b, color, next);
        atari = next;
    }
}

/* FastBoard::check_winning_ladder: playing vtx puts an opponent string of
 * two liberties in atari and its escape (with two empty neighbours) loses. */
static int gb_winning_ladder(const int8_t *board, int color, int vtx) {
    int nb[4], m = gb_nbrs(vtx, nb);
    for (int k = 0; k < m; ++k) {
        int r = nb[k];
        if (board[r] != 1 - color || gb_libs(board, r) != 2) continue;
        if (gb_self_atari(board, color, vtx)) continue;
        int8_t b[OR_POINTS];
        memcpy(b, board, sizeof b);
        gb_play(b, color, vtx);
        int esc;
        if (gb_liberties(b, r, 2, &esc) < 1) continue;
        if (gb_count_empty(b, esc) == 2 && gb_losing_ladder(b, 1 - color, esc, 0)) return 1;
    }
    return 0;
}

void or_gather_planes(const int8_t *squares, int to_move, const int32_t *moves, int which, int nplanes,
                      uint8_t *planes) {
    memset(planes, 0, (size_t)nplanes * OR_POINTS);
    int libs_of[OR_POINTS];
    uint8_t done[OR_POINTS];
    memset(done, 0, sizeof done);
    for (int p = 0; p < OR_POINTS; ++p) {
        if (squares[p] == GB_EMPTY || done[p]) continue;
        int list[OR_POINTS], n;
        uint8_t in[OR_POINTS];
        memset(in, 0, sizeof in);
        int l = gb_string(squares, p, in, list, &n);
        for (int i = 0; i < n; ++i) { libs_of[list[i]] = l; done[list[i]] = 1; }
    }
    /* policy: own libs 1,2,3,4,5+ at 3..7, opponent's at 8..12, after-move
     * 1..5,6+ at 13..18, opponent's after-move 1..5,6+ at 19..24, ladder 25,
     * ladder win 26, ko 27, last move 28, the move before 29, white stones
     * when white has komi 30, third line 31.  value: libs 1..5,6+ at 3..8 /
     * 9..14, after-move 1..5,6+ at 15..20 / 21..26, ladder 27, ladder win 28,
     * komi 29, third line 30, ko 31. */
    const int lib_cap = which == 0 ? 5 : 6;
    const int opp_lib0 = which == 0 ? 8 : 9;
    const int after0 = which == 0 ? 13 : 15;
    const int oafter0 = which == 0 ? 19 : 21;
    const int p_ladder = which == 0 ? 25 : 27, p_win = which == 0 ? 26 : 28;
    const int p_komi = which == 0 ? 30 : 29, p_line3 = which == 0 ? 31 : 30;
    const int p_ko = which == 0 ? 27 : 31;
#define SETP(plane, p) do { if ((plane) < nplanes) planes[(size_t)(plane) * OR_POINTS + (p)] = 1; } while (0)
    for (int p = 0; p < OR_POINTS; ++p) {
        int c = squares[p], x = p % 19, y = p / 19;
        if (x == 2 || x == 16 || y == 2 || y == 16) SETP(p_line3, p);
        if (c != GB_EMPTY) {
            int mine = c == to_move;
            if (c == 1 && moves && moves[3]) SETP(p_komi, p);
            SETP(mine ? 1 : 2, p);
            int l = libs_of[p];
            if (l >= 1) SETP((mine ? 3 : opp_lib0) + (l >= lib_cap ? lib_cap : l) - 1, p);
        } else {
            SETP(0, p);
            int al = gb_after(squares, to_move, p);
            int at = gb_after(squares, 1 - to_move, p);
            if (al >= 1) SETP(after0 + (al >= 6 ? 5 : al - 1), p);
            if (at >= 1) SETP(oafter0 + (at >= 6 ? 5 : at - 1), p);
            if (nplanes > 24) {
                if (gb_count_empty(squares, p) == 2 && gb_saving_size(squares, to_move, p) > 0 &&
                    gb_losing_ladder(squares, to_move, p, 0))
                    SETP(p_ladder, p);
                if (gb_winning_ladder(squares, to_move, p)) SETP(p_win, p);
            }
        }
    }
    if (moves) {
        if (moves[0] >= 0 && which == 0) {
            SETP(28, moves[0]);
            if (moves[1] >= 0) SETP(29, moves[1]);
        }
        if (moves[2] >= 0) SETP(p_ko, moves[2]);
    }
#undef SETP
}

int or_random_board(uint64_t seed, int k, int8_t *squares) {
    uint64_t s = seed * 0x9E3779B97F4A7C15ull + 0x5851F42D4C957F2Dull;
    memset(squares, GB_EMPTY, OR_POINTS);
    int color = 0;
    for (int mv = 0; mv < k; ++mv) {
        /* uniform over the legal points: draw empty points without
         * replacement until one is not a suicide */
        int cand[OR_POINTS], nc = 0, p = -1;
        for (int q = 0; q < OR_POINTS; ++q)
            if (squares[q] == GB_EMPTY) cand[nc++] = q;
        while (nc > 0) {
            int j = (int)(splitmix64(&s) % (uint64_t)nc);
            int q = cand[j];
            if (gb_after(squares, color, q) > 0) { p = q; break; }
            cand[j] = cand[--nc];
        }
        if (p < 0) break;
        int nb[4], m = gb_nbrs(p, nb);
        squares[p] = (int8_t)color;
        for (int j = 0; j < m; ++j) {
            int r = nb[j];
            if (squares[r] == 1 - color && gb_libs(squares, r) == 0) {
                uint8_t in[OR_POINTS];
                int list[OR_POINTS], n;
                memset(in, 0, sizeof in);
                gb_string(squares, r, in, list, &n);
                for (int i = 0; i < n; ++i) squares[list[i]] = GB_EMPTY;
            }
        }
        color = 1 - color;
    }
    return color;
}

/* A config-0/1/2 position: from the empty board, k ~ U[0, kmax] moves, each
 * uniform over the legal non-pass moves (empty, not the simple-ko point,
 * not a suicide: FastState::generate_moves, FastState.cpp:57-73), passing
 * only when nothing else is legal.  Captures as FullBoard::update_board
 * (FullBoard.cpp:130-201) makes them; the ko point is the captured point
 * when the stone was played into an opponent eye and captured exactly one
 * stone (FullBoard.cpp:149-150, 192-197).  Writes squares[361] and
 * moves[4] = last move, the move before it (-1 none or pass), ko point
 * (-1 none), white-has-komi flag (1: komi 7.5 goes to white); returns the
 * side to move.  Uses its own splitmix64 stream, so the positions are the
 * same on every host. */
int or_config_board(uint64_t seed, int kmax, int8_t *squares, int32_t *moves) {
    uint64_t s = seed * 0xD1B54A32D192ED03ull + 0x2545F4914F6CDD1Dull;
    memset(squares, GB_EMPTY, OR_POINTS);
    int k = (int)(splitmix64(&s) % (uint64_t)(kmax + 1));
    int color = 0, ko = -1, last = -1, prev = -1;
    for (int mv = 0; mv < k; ++mv) {
        int cand[OR_POINTS], nc = 0, p = -1;
        for (int q = 0; q < OR_POINTS; ++q)
            if (squares[q] == GB_EMPTY && q != ko) cand[nc++] = q;
        while (nc > 0) {
            int j = (int)(splitmix64(&s) % (uint64_t)nc);
            int q = cand[j];
            if (gb_after(squares, color, q) > 0) { p = q; break; }
            cand[j] = cand[--nc];
        }
        prev = last;
        last = p;
        ko = -1;
        if (p >= 0) {
            int nb[4], m = gb_nbrs(p, nb), eye = 1, captured = 0, csq = -1;
            for (int j = 0; j < m; ++j) eye &= squares[nb[j]] == 1 - color;
            squares[p] = (int8_t)color;
            for (int j = 0; j < m; ++j) {
                int r = nb[j];
                if (squares[r] == 1 - color && gb_libs(squares, r) == 0) {
                    uint8_t in[OR_POINTS];
                    int list[OR_POINTS], n;
                    memset(in, 0, sizeof in);
                    gb_string(squares, r, in, list, &n);
                    for (int i = 0; i < n; ++i) squares[list[i]] = GB_EMPTY;
                    captured += n;
                    csq = r;
                }
            }
            if (captured == 1 && eye) ko = csq;
        }
        color = 1 - color;
    }
    moves[0] = last;
    moves[1] = prev;
    moves[2] = ko;
    moves[3] = 1;
    return color;
}

/* Positions start .. start + n - 1 of stream `base` (position i from seed
 * base + i, as or_config_board): squares [n][361], moves [n][4], to_move [n]. */
void or_config_boards(uint64_t base, int start, int n, int kmax, int8_t *squares, int32_t *moves,
                      int8_t *to_move) {
    for (int i = 0; i < n; ++i)
        to_move[i] = (int8_t)or_config_board(base + (uint64_t)(start + i), kmax, squares + (size_t)i * OR_POINTS,
                                             moves + (size_t)i * 4);
}

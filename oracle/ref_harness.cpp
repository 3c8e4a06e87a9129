// ref_harness.cpp -- drives the reference engine's own CPU/BLAS code.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile from the reference
// sources where they lie (read-only) into oracle/_ref/; never shipped and
// never linked into the product.  It produces the golden fixtures in
// tests/golden (positions, gathered planes, reference outputs) and times the
// reference CPU path during development.
//
// The reference's Network.cpp is compiled inside this translation unit so
// that its private helpers (feature gather, *_internal forwards) and its
// BLAS templates convolve<>/innerproduct<> (Network.cpp:345-423) can be
// called directly.  The weight arrays it declares extern
// (Network.cpp:82-137) are defined here and filled, at static-init time,
// from the file named by LEELA_REF_WEIGHTS (policy arrays then value arrays,
// each conv as W then b, in declaration order).
//
// Commands (all positions are regenerated from the seed, see make_position):
//   gen      N SEED OUT          positions: planes, squares, metadata
//   refexact N SEED ROT OUT      reference get_scored_moves(DIRECT, ROT) and
//                                get_value_internal(ROT) with the loaded weights
//   config   N SEED ROT WP WV OUT  config-1 shaped nets (24->128 5x5, 11x 3x3,
//                                1x1 head, ReLU, tanh) through the reference's
//                                im2col + cblas_sgemm; WP/WV = flat weight files
//   elucheck WP                  bit-compare the harness conv (ELU) with the
//                                reference convolve<5,24,128>/<3,128,128>
//   mcowner  N SEED PLAYOUTS THREADS OUT   Playout::mc_owner labels
//   mcfile   SQ TM MV N PLAYOUTS THREADS OUT  Playout::mc_owner labels of N
//                                positions given as files: squares int8
//                                [N][361], to_move int8 [N], moves int32
//                                [N][4] (last, before last, ko point, komi flag)
//   time     N SEED THREADS SECS WP WV     reference CPU pos/s, config-1 nets
#include <algorithm>
#include <array>
#include <climits>
#include <condition_variable>
#include <cstddef>
#include <functional>
#include <future>
#include <map>
#include <mutex>
#include <queue>
#include <sstream>
#include <tuple>
#include <assert.h>
#include <sys/time.h>
#include <time.h>
#include <atomic>
#include <bitset>
#include <cassert>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <list>
#include <memory>
#include <set>
#include <string>
#include <thread>
#include <vector>

#define private public
#define protected public
#include "Network.cpp"
#undef private
#undef protected

#include "GTP.h"
#include "GameState.h"
#include "Playout.h"
#include "Random.h"
#include "Zobrist.h"

// ------------------------------------------------------------ weights

namespace {
std::vector<float> &weight_blob() {
    static std::vector<float> blob;
    static bool loaded = false;
    if (!loaded) {
        loaded = true;
        const char *path = std::getenv("LEELA_REF_WEIGHTS");
        if (path) {
            std::ifstream f(path, std::ios::binary);
            f.seekg(0, std::ios::end);
            size_t bytes = (size_t)f.tellg();
            f.seekg(0);
            blob.resize(bytes / sizeof(float));
            f.read(reinterpret_cast<char *>(blob.data()), (std::streamsize)bytes);
        }
    }
    return blob;
}
size_t &weight_cursor() {
    static size_t cur = 0;
    return cur;
}
template <size_t N> std::array<float, N> next_weights() {
    std::array<float, N> a{};
    auto &blob = weight_blob();
    size_t &cur = weight_cursor();
    if (cur + N <= blob.size()) std::copy(blob.begin() + cur, blob.begin() + cur + N, a.begin());
    cur += N;
    return a;
}
}  // namespace

#define W(name, n) extern const std::array<float, n> name = next_weights<n>();
W(conv1_w, 76800) W(conv1_b, 96) W(conv2_w, 110592) W(conv2_b, 128)
W(conv3_w, 147456) W(conv3_b, 128) W(conv4_w, 147456) W(conv4_b, 128)
W(conv5_w, 147456) W(conv5_b, 128) W(conv6_w, 147456) W(conv6_b, 128)
W(conv7_w, 147456) W(conv7_b, 128) W(conv8_w, 147456) W(conv8_b, 128)
W(conv9_w, 147456) W(conv9_b, 128) W(conv10_w, 147456) W(conv10_b, 128)
W(conv11_w, 147456) W(conv11_b, 128) W(conv12_w, 147456) W(conv12_b, 128)
W(conv13_w, 1152) W(conv13_b, 1)
W(val_conv1_w, 51200) W(val_conv1_b, 64) W(val_conv2_w, 36864) W(val_conv2_b, 64)
W(val_conv3_w, 36864) W(val_conv3_b, 64) W(val_conv4_w, 36864) W(val_conv4_b, 64)
W(val_conv5_w, 36864) W(val_conv5_b, 64) W(val_conv6_w, 36864) W(val_conv6_b, 64)
W(val_conv7_w, 36864) W(val_conv7_b, 64) W(val_conv8_w, 36864) W(val_conv8_b, 64)
W(val_conv9_w, 36864) W(val_conv9_b, 64) W(val_conv10_w, 36864) W(val_conv10_b, 64)
W(val_conv11_w, 36864) W(val_conv11_b, 64) W(val_conv12_w, 576) W(val_conv12_b, 1)
W(val_ip13_w, 92416) W(val_ip13_b, 256) W(val_ip14_w, 256) W(val_ip14_b, 1)
#undef W

// ------------------------------------------------------------ positions

namespace {

void init_engine(int threads) {
    GTP::setup_default_parameters();
    cfg_num_threads = threads;
    thread_pool.initialize(cfg_num_threads);
    std::unique_ptr<Random> rng(new Random(5489));
    Zobrist::init_zobrist(*rng);
    openblas_set_num_threads(1);
}

// Synthetic position i of a seeded set: an empty 19x19 board, komi 7.5,
// then k ~ U[0,250] moves, each uniform over the legal non-pass moves
// (FastState::generate_moves: empty, not the simple-ko point, not suicide);
// a pass only when no other move is legal.  The draws come from one
// splitmix64 stream per set, in position order.  (The reference's own
// xoroshiro128+ `Random(seed)` cannot be used here: Random::seedrandom
// (Random.cpp:55-61) maps seed 0 to the all-zero state, which only ever
// returns 0.)
struct PositionStream {
    explicit PositionStream(int seed) : s((uint64_t)seed) {}
    uint64_t next64() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    // Uniform integer in [0, n): the high 32 bits scaled by n.
    uint32_t below(uint32_t n) { return (uint32_t)(((next64() >> 32) * (uint64_t)n) >> 32); }
    GameState next(int *k_out) {
        GameState g;
        g.init_game(19, 7.5f);
        int k = (int)below(251);
        for (int m = 0; m < k; ++m) {
            std::vector<int> moves = g.generate_moves(g.get_to_move());
            moves.erase(std::remove(moves.begin(), moves.end(), +FastBoard::PASS), moves.end());
            if (moves.empty()) {
                g.play_pass();
            } else {
                g.play_move(moves[below((uint32_t)moves.size())]);
            }
        }
        *k_out = k;
        return g;
    }
    uint64_t s;
};

void planes_to_bytes(const Network::NNPlanes &planes, int nplanes, int rotation,
                     std::vector<uint8_t> &out) {
    for (int c = 0; c < nplanes; ++c)
        for (int i = 0; i < 361; ++i)
            out.push_back((uint8_t)planes[c][Network::rotate_nn_idx(i, rotation)]);
}

FILE *open_out(const std::string &prefix, const char *ext) {
    std::string p = prefix + ext;
    FILE *f = std::fopen(p.c_str(), "wb");
    if (!f) {
        std::perror(p.c_str());
        std::exit(2);
    }
    return f;
}

std::vector<float> read_floats(const char *path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        std::fprintf(stderr, "cannot open %s\n", path);
        std::exit(2);
    }
    f.seekg(0, std::ios::end);
    size_t bytes = (size_t)f.tellg();
    f.seekg(0);
    std::vector<float> v(bytes / sizeof(float));
    f.read(reinterpret_cast<char *>(v.data()), (std::streamsize)bytes);
    return v;
}

// ------------------------------------------------ config-1 shaped nets
//
// The reference hard-codes ELU in convolve<> and innerproduct<>
// (Network.cpp:382-392, 411-422).  The config-1 nets use ReLU and no
// activation after the last conv, so this harness runs the same im2col<>
// (Im2Col.h) and the same cblas_sgemm call shape, with the bias and the
// activation applied afterwards; elucheck verifies that with ELU this equals
// the reference template bit for bit.

enum Act { ACT_ELU = 0, ACT_RELU = 1, ACT_NONE = 2 };

inline float apply_act(float v, int act) {
    if (act == ACT_ELU) return (v > 0.0f) ? v : 1.0f * (std::exp(v) - 1.0f);
    if (act == ACT_RELU) return (v > 0.0f) ? v : 0.0f;
    return v;
}

template <unsigned C, unsigned K>
void conv_act(std::vector<float> &in, const float *w, const float *b, unsigned outputs, int act,
              std::vector<float> &out) {
    std::vector<float> col(C * K * K * 361);
    im2col<C, K>(in, col);
    cblas_sgemm(CblasRowMajor, CblasNoTrans, CblasNoTrans, outputs, 361, C * K * K, 1.0f, w,
                C * K * K, &col[0], 361, 0.0f, &out[0], 361);
    for (unsigned o = 0; o < outputs; ++o)
        for (unsigned p = 0; p < 361; ++p) out[o * 361 + p] = apply_act(b[o] + out[o * 361 + p], act);
}

// Flat layout: per conv W[O][C][k][k], b[O]; then W1[256][361], b1, W2[256], b2.
struct Config1Net {
    std::vector<float> w;
    bool value;
    // logits (policy: 361) or pre-tanh scalar + mapped value (value net).
    void run(const std::vector<uint8_t> &planes24, float *out) const {
        std::vector<float> a(128 * 361, 0.0f), b(128 * 361, 0.0f);
        for (size_t i = 0; i < 24 * 361; ++i) a[i] = (float)planes24[i];
        size_t off = 0;
        conv_act<24, 5>(a, &w[off], &w[off + 76800], 128, ACT_RELU, b);
        off += 76800 + 128;
        std::swap(a, b);
        for (int l = 0; l < 11; ++l) {
            conv_act<128, 3>(a, &w[off], &w[off + 147456], 128, ACT_RELU, b);
            off += 147456 + 128;
            std::swap(a, b);
        }
        conv_act<128, 1>(a, &w[off], &w[off + 128], 1, ACT_NONE, b);
        off += 128 + 1;
        if (!value) {
            std::copy(b.begin(), b.begin() + 361, out);
            return;
        }
        std::vector<float> hidden(256), y(1);
        cblas_sgemv(CblasRowMajor, CblasNoTrans, 256, 361, 1.0f, &w[off], 361, &b[0], 1, 0.0f,
                    &hidden[0], 1);
        const float *b1 = &w[off + 256 * 361];
        for (int o = 0; o < 256; ++o) hidden[o] = apply_act(b1[o] + hidden[o], ACT_RELU);
        const float *w2 = b1 + 256;
        cblas_sgemv(CblasRowMajor, CblasNoTrans, 1, 256, 1.0f, w2, 256, &hidden[0], 1, 0.0f, &y[0], 1);
        float x = w2[256] + y[0];
        out[0] = x;
        out[1] = std::tanh(x);
    }
};

const size_t kConfig1Policy = 76800 + 128 + 11 * (147456 + 128) + 128 + 1;
const size_t kConfig1Value = kConfig1Policy + 256 * 361 + 256 + 256 + 1;

int cmd_gen(int n, int seed, const std::string &out) {
    PositionStream ps(seed);
    FILE *fp = open_out(out, ".planes_p"), *fv = open_out(out, ".planes_v");
    FILE *fs = open_out(out, ".squares"), *fm = open_out(out, ".meta");
    FILE *fmv = open_out(out, ".moves");
    // a board vertex as a point index y*19+x, -1 for none (vertex <= 0)
    auto point_of = [](GameState &g, int v) -> int32_t {
        if (v <= 0) return -1;
        std::pair<int, int> xy = g.board.get_xy(v);
        return xy.second * 19 + xy.first;
    };
    for (int i = 0; i < n; ++i) {
        int k;
        GameState g = ps.next(&k);
        Network::NNPlanes pp, pv;
        Network::BoardPlane *ladder = nullptr;
        Network::gather_features_policy(&g, pp, &ladder);
        Network::gather_features_value(&g, pv);
        std::vector<uint8_t> bp, bv;
        planes_to_bytes(pp, 32, 0, bp);
        planes_to_bytes(pv, 32, 0, bv);
        std::fwrite(bp.data(), 1, bp.size(), fp);
        std::fwrite(bv.data(), 1, bv.size(), fv);
        int8_t sq[361];
        for (int j = 0; j < 361; ++j) sq[j] = (int8_t)g.board.get_square(g.board.get_vertex(j % 19, j / 19));
        std::fwrite(sq, 1, 361, fs);
        int32_t meta[4] = {g.get_to_move(), (int32_t)g.get_movenum(), k, g.get_komove()};
        std::fwrite(meta, sizeof(int32_t), 4, fm);
        // what the gather reads besides the board: last move, the move before
        // it, the ko point, and whether white has komi (|komi| > 0.75)
        int32_t mv[4] = {point_of(g, g.get_last_move()), point_of(g, g.get_prevlast_move()),
                         point_of(g, g.get_komove()), std::fabs(g.get_komi()) > 0.75f ? 1 : 0};
        std::fwrite(mv, sizeof(int32_t), 4, fmv);
    }
    std::fclose(fp); std::fclose(fv); std::fclose(fs); std::fclose(fm); std::fclose(fmv);
    return 0;
}

// Reference-exact nets: 32 planes, ELU everywhere, 3x3 heads, policy
// 32->96->128x10->1 and value 32->64x10->1 + FC 361->256->1, (1+tanh)/2.
int cmd_refexact(int n, int seed, int rot, const std::string &out) {
    PositionStream ps(seed);
    FILE *fprob = open_out(out, ".probs"), *flog = open_out(out, ".logits");
    FILE *fval = open_out(out, ".value");
    for (int i = 0; i < n; ++i) {
        int k;
        GameState g = ps.next(&k);
        // Netresult from the public entry point, scattered to board order
        // (-1 for occupied points); ladder pruning included.
        Network::Netresult res = Network::get_scored_moves(&g, Network::DIRECT, rot);
        std::vector<float> probs(361, -1.0f);
        for (auto &sn : res) {
            auto xy = g.board.get_xy(sn.second);
            probs[xy.second * 19 + xy.first] = sn.first;
        }
        std::fwrite(probs.data(), sizeof(float), 361, fprob);
        // Raw policy output (after the head ELU) in network order for the
        // same rotation: the reference's own convolve<> chain
        // (Network.cpp:783-807).
        Network::NNPlanes planes;
        Network::BoardPlane *ladder = nullptr;
        Network::gather_features_policy(&g, planes, &ladder);
        std::vector<float> input(Network::MAX_CHANNELS * 361, 0.0f), output(Network::MAX_CHANNELS * 361);
        for (int c = 0; c < 32; ++c)
            for (int j = 0; j < 361; ++j) input[c * 361 + j] = (float)planes[c][Network::rotate_nn_idx(j, rot)];
        convolve<5, 32, 96>(input, conv1_w, conv1_b, output); std::swap(input, output);
        convolve<3, 96, 128>(input, conv2_w, conv2_b, output); std::swap(input, output);
        convolve<3, 128, 128>(input, conv3_w, conv3_b, output); std::swap(input, output);
        convolve<3, 128, 128>(input, conv4_w, conv4_b, output); std::swap(input, output);
        convolve<3, 128, 128>(input, conv5_w, conv5_b, output); std::swap(input, output);
        convolve<3, 128, 128>(input, conv6_w, conv6_b, output); std::swap(input, output);
        convolve<3, 128, 128>(input, conv7_w, conv7_b, output); std::swap(input, output);
        convolve<3, 128, 128>(input, conv8_w, conv8_b, output); std::swap(input, output);
        convolve<3, 128, 128>(input, conv9_w, conv9_b, output); std::swap(input, output);
        convolve<3, 128, 128>(input, conv10_w, conv10_b, output); std::swap(input, output);
        convolve<3, 128, 128>(input, conv11_w, conv11_b, output); std::swap(input, output);
        convolve<3, 128, 128>(input, conv12_w, conv12_b, output); std::swap(input, output);
        convolve<3, 128, 1>(input, conv13_w, conv13_b, output);
        std::fwrite(output.data(), sizeof(float), 361, flog);
        Network::NNPlanes vplanes;
        Network::gather_features_value(&g, vplanes);
        float v = Network::get_value_internal(&g, vplanes, rot);
        std::fwrite(&v, sizeof(float), 1, fval);
    }
    std::fclose(fprob); std::fclose(flog); std::fclose(fval);
    return 0;
}

int cmd_config(int n, int seed, int rot, const char *wp, const char *wv, const std::string &out) {
    Config1Net pol{read_floats(wp), false}, val{read_floats(wv), true};
    if (pol.w.size() != kConfig1Policy || val.w.size() != kConfig1Value) {
        std::fprintf(stderr, "config-1 weight sizes %zu/%zu, want %zu/%zu\n", pol.w.size(),
                     val.w.size(), kConfig1Policy, kConfig1Value);
        return 2;
    }
    PositionStream ps(seed);
    FILE *flog = open_out(out, ".logits"), *fprob = open_out(out, ".probs");
    FILE *fval = open_out(out, ".value");
    for (int i = 0; i < n; ++i) {
        int k;
        GameState g = ps.next(&k);
        Network::NNPlanes pp, pv;
        Network::BoardPlane *ladder = nullptr;
        Network::gather_features_policy(&g, pp, &ladder);
        Network::gather_features_value(&g, pv);
        std::vector<uint8_t> bp, bv;
        planes_to_bytes(pp, 24, rot, bp);
        planes_to_bytes(pv, 24, rot, bv);
        std::vector<float> logits(361), probs(361);
        pol.run(bp, logits.data());
        // The reference softmax at temperature 1 (Network.cpp:450-469).
        Network::softmax(logits, probs, 1.0f);
        float vo[2];
        val.run(bv, vo);
        std::fwrite(logits.data(), sizeof(float), 361, flog);
        std::fwrite(probs.data(), sizeof(float), 361, fprob);
        std::fwrite(vo, sizeof(float), 2, fval);
    }
    std::fclose(flog); std::fclose(fprob); std::fclose(fval);
    return 0;
}

int cmd_elucheck(const char *wp) {
    std::vector<float> w = read_floats(wp);
    if (w.size() != kConfig1Policy) return 2;
    PositionStream ps(0);
    int k;
    ps.next(&k);
    GameState g = ps.next(&k);
    Network::NNPlanes pp;
    Network::BoardPlane *ladder = nullptr;
    Network::gather_features_policy(&g, pp, &ladder);
    std::vector<float> a(128 * 361, 0.0f);
    for (int c = 0; c < 24; ++c)
        for (int j = 0; j < 361; ++j) a[c * 361 + j] = (float)pp[c][j];
    auto w1 = std::make_unique<std::array<float, 76800>>();
    auto b1 = std::make_unique<std::array<float, 128>>();
    std::copy(w.begin(), w.begin() + 76800, w1->begin());
    std::copy(w.begin() + 76800, w.begin() + 76800 + 128, b1->begin());
    std::vector<float> ref(128 * 361), mine(128 * 361);
    std::vector<float> a2 = a;
    convolve<5, 24, 128>(a2, *w1, *b1, ref);
    conv_act<24, 5>(a, w1->data(), b1->data(), 128, ACT_ELU, mine);
    size_t diff = 0;
    for (size_t i = 0; i < ref.size(); ++i) diff += (std::memcmp(&ref[i], &mine[i], 4) != 0);
    auto w3 = std::make_unique<std::array<float, 147456>>();
    auto b3 = std::make_unique<std::array<float, 128>>();
    size_t off = 76800 + 128;
    std::copy(w.begin() + off, w.begin() + off + 147456, w3->begin());
    std::copy(w.begin() + off + 147456, w.begin() + off + 147456 + 128, b3->begin());
    std::vector<float> r3(128 * 361), m3(128 * 361);
    std::vector<float> in3 = ref, in3b = ref;
    convolve<3, 128, 128>(in3, *w3, *b3, r3);
    conv_act<128, 3>(in3b, w3->data(), b3->data(), 128, ACT_ELU, m3);
    for (size_t i = 0; i < r3.size(); ++i) diff += (std::memcmp(&r3[i], &m3[i], 4) != 0);
    std::printf("elucheck mismatches %zu\n", diff);
    return diff == 0 ? 0 : 1;
}

int cmd_mcowner(int n, int seed, int playouts, const std::string &out) {
    PositionStream ps(seed);
    FILE *f = open_out(out, ".mcowner");
    for (int i = 0; i < n; ++i) {
        int k;
        GameState g = ps.next(&k);
        FastState fs = g;
        float w = Playout::mc_owner(fs, playouts);
        std::fwrite(&w, sizeof(float), 1, f);
    }
    std::fclose(f);
    return 0;
}

// Labels for positions that come as boards (the oracle's generator at scale,
// where replaying every move list here would be the slow part).  Each
// position is set up by placing its stones on an empty board: placing the
// stones of a legal position in any order captures nothing and is never a
// suicide (a partial string always touches an empty point: one of its final
// liberties, or a stone of its string not yet placed), so FastState's own
// play_move builds the same strings, liberties and hashes.  The side to
// move, the ko point and the last two moves are then set as given.
// Positions are spread over THREADS caller threads; each calls mc_owner with
// cfg_num_threads = 1, so every label is exactly PLAYOUTS playouts, run on
// the engine's thread pool (THREADS workers).
int cmd_mcfile(const char *sqf, const char *tmf, const char *mvf, int n, int playouts, int threads,
               const std::string &out) {
    auto read_all = [](const char *path, size_t bytes) {
        std::vector<char> v(bytes);
        std::ifstream f(path, std::ios::binary);
        if (!f || !f.read(v.data(), (std::streamsize)bytes)) {
            std::fprintf(stderr, "cannot read %zu bytes from %s\n", bytes, path);
            std::exit(2);
        }
        return v;
    };
    const std::vector<char> sq = read_all(sqf, (size_t)n * 361);
    const std::vector<char> tm = read_all(tmf, (size_t)n);
    const std::vector<char> mvb = read_all(mvf, (size_t)n * 16);
    const int32_t *mv = reinterpret_cast<const int32_t *>(mvb.data());
    std::vector<float> w(n);
    cfg_num_threads = 1;
    std::atomic<int> next{0};
    std::vector<std::thread> ts;
    for (int t = 0; t < threads; ++t)
        ts.emplace_back([&]() {
            for (int i = next.fetch_add(1); i < n; i = next.fetch_add(1)) {
                FastState fs;
                fs.init_game(19, 7.5f);
                auto vtx = [&](int p) { return p < 0 ? 0 : fs.board.get_vertex(p % 19, p / 19); };
                for (int p = 0; p < 361; ++p) {
                    const int c = sq[(size_t)i * 361 + p];
                    if (c == FastBoard::BLACK || c == FastBoard::WHITE) fs.play_move(c, vtx(p));
                }
                fs.set_to_move(tm[i]);
                fs.m_lastmove = vtx(mv[i * 4 + 0]);
                fs.m_onebutlastmove = vtx(mv[i * 4 + 1]);
                fs.m_komove = vtx(mv[i * 4 + 2]);
                fs.m_passes = 0;
                fs.m_last_was_capture = false;
                w[i] = Playout::mc_owner(fs, playouts);
            }
        });
    for (auto &th : ts) th.join();
    FILE *f = open_out(out, ".mcowner");
    std::fwrite(w.data(), sizeof(float), (size_t)n, f);
    std::fclose(f);
    return 0;
}

int cmd_time(int n, int seed, int threads, double secs, const char *wp, const char *wv) {
    Config1Net pol{read_floats(wp), false}, val{read_floats(wv), true};
    PositionStream ps(seed);
    std::vector<std::vector<uint8_t>> bp(n), bv(n);
    for (int i = 0; i < n; ++i) {
        int k;
        GameState g = ps.next(&k);
        Network::NNPlanes pp, pv;
        Network::BoardPlane *ladder = nullptr;
        Network::gather_features_policy(&g, pp, &ladder);
        Network::gather_features_value(&g, pv);
        planes_to_bytes(pp, 24, 0, bp[i]);
        planes_to_bytes(pv, 24, 0, bv[i]);
    }
    std::atomic<long> done{0};
    std::atomic<bool> stop{false};
    auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> ts;
    for (int t = 0; t < threads; ++t)
        ts.emplace_back([&, t]() {
            float lo[361], vo[2];
            for (long i = t; !stop.load(); i += threads) {
                pol.run(bp[i % n], lo);
                val.run(bv[i % n], vo);
                done.fetch_add(1);
            }
        });
    std::this_thread::sleep_for(std::chrono::duration<double>(secs));
    stop = true;
    for (auto &th : ts) th.join();
    double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("{\"pairs\": %ld, \"seconds\": %.3f, \"threads\": %d, \"pair_pos_per_s\": %.2f}\n",
                done.load(), el, threads, done.load() / el);
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: ref_harness gen|refexact|config|elucheck|mcowner|mcfile|time ...\n");
        return 2;
    }
    std::string cmd = argv[1];
    int threads = 1;
    if (cmd == "mcowner" && argc >= 7) threads = std::atoi(argv[5]);
    if (cmd == "time" && argc >= 5) threads = std::atoi(argv[4]);
    if (cmd == "mcfile" && argc >= 8) threads = std::atoi(argv[7]);
    init_engine(threads);
    if (cmd == "gen" && argc == 5) return cmd_gen(std::atoi(argv[2]), std::atoi(argv[3]), argv[4]);
    if (cmd == "refexact" && argc == 6)
        return cmd_refexact(std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4]), argv[5]);
    if (cmd == "config" && argc == 8)
        return cmd_config(std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4]), argv[5], argv[6],
                          argv[7]);
    if (cmd == "elucheck" && argc == 3) return cmd_elucheck(argv[2]);
    if (cmd == "mcowner" && argc == 7)
        return cmd_mcowner(std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4]), argv[6]);
    if (cmd == "mcfile" && argc == 9)
        return cmd_mcfile(argv[2], argv[3], argv[4], std::atoi(argv[5]), std::atoi(argv[6]), threads, argv[8]);
    if (cmd == "time" && argc == 8)
        return cmd_time(std::atoi(argv[2]), std::atoi(argv[3]), threads, std::atof(argv[5]), argv[6],
                        argv[7]);
    std::fprintf(stderr, "bad arguments\n");
    return 2;
}

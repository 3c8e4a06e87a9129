// search_driver.cpp -- the engine's own UCT search, in its OpenCL
// configuration, evaluating through the GB300 backend
// (leela_gb300/integration/opencl_gb300.cpp) and the CPU stand-in of the C
// ABI (fake_lg.cpp).
//
// TEST INFRASTRUCTURE ONLY (tests/test_search_integration.py).  The
// engine's sources are compiled unmodified where they lie; this file
// supplies what the missing weight files would (Network.cpp:54-137, OpenCL
// shapes: policy 32->128->192x11->1, value 32->64x10->1 + FC 361->256->1,
// seeded He-normal) and a main that runs one search:
//
//   search_driver PLAYOUTS THREADS
//
// and prints one line of counters the test checks.
#include <array>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>
#include <vector>
#include <dlfcn.h>

#include "GTP.h"
#include "GameState.h"
#include "Network.h"
#include "Random.h"
#include "ThreadPool.h"
#include "Utils.h"
#include "UCTSearch.h"
#include "Zobrist.h"
#define private public
#include "OpenCL.h"
#undef private
#include "leela_oracle.h"

extern "C" long long fake_lg_submitted();
extern "C" long long fake_lg_sync_calls();

namespace {
or_net shape(bool value) {
    // c_in, width1, width, n3x3, head_k, act (ELU), act_head, value_head, fc_hidden, value_map
    return value ? or_net{32, 64, 64, 10, 3, 0, 1, 1, 256, 1} : or_net{32, 128, 192, 11, 3, 0, 1, 0, 0, 0};
}
const std::vector<float> &flat(bool value) {
    static std::vector<float> w[2];
    std::vector<float> &v = w[value ? 1 : 0];
    if (v.empty()) {
        or_net n = shape(value);
        v.resize(or_weight_count(&n));
        or_he_weights(&n, value ? 2 : 1, v.data());
    }
    return v;
}
size_t cursor[2] = {0, 0};
template <size_t N> std::array<float, N> take(bool value) {
    std::array<float, N> a{};
    const std::vector<float> &v = flat(value);
    size_t &c = cursor[value ? 1 : 0];
    for (size_t i = 0; i < N && c + i < v.size(); ++i) a[i] = v[c + i];
    c += N;
    return a;
}
}  // namespace

#define P(name, n) extern const std::array<float, n> name = take<n>(false);
#define V(name, n) extern const std::array<float, n> name = take<n>(true);
P(conv1_w, 102400) P(conv1_b, 128) P(conv2_w, 221184) P(conv2_b, 192)
P(conv3_w, 331776) P(conv3_b, 192) P(conv4_w, 331776) P(conv4_b, 192)
P(conv5_w, 331776) P(conv5_b, 192) P(conv6_w, 331776) P(conv6_b, 192)
P(conv7_w, 331776) P(conv7_b, 192) P(conv8_w, 331776) P(conv8_b, 192)
P(conv9_w, 331776) P(conv9_b, 192) P(conv10_w, 331776) P(conv10_b, 192)
P(conv11_w, 331776) P(conv11_b, 192) P(conv12_w, 331776) P(conv12_b, 192)
P(conv13_w, 1728) P(conv13_b, 1)
V(val_conv1_w, 51200) V(val_conv1_b, 64) V(val_conv2_w, 36864) V(val_conv2_b, 64)
V(val_conv3_w, 36864) V(val_conv3_b, 64) V(val_conv4_w, 36864) V(val_conv4_b, 64)
V(val_conv5_w, 36864) V(val_conv5_b, 64) V(val_conv6_w, 36864) V(val_conv6_b, 64)
V(val_conv7_w, 36864) V(val_conv7_b, 64) V(val_conv8_w, 36864) V(val_conv8_b, 64)
V(val_conv9_w, 36864) V(val_conv9_b, 64) V(val_conv10_w, 36864) V(val_conv10_b, 64)
V(val_conv11_w, 36864) V(val_conv11_b, 64) V(val_conv12_w, 576) V(val_conv12_b, 1)
V(val_ip13_w, 92416) V(val_ip13_b, 256) V(val_ip14_w, 256) V(val_ip14_b, 1)
#undef P
#undef V

int main(int argc, char **argv) {
    const int playouts = argc > 1 ? std::atoi(argv[1]) : 300;
    const int threads = argc > 2 ? std::atoi(argv[2]) : 4;
    if (const char *blas = std::getenv("LEELA_OPENBLAS")) {
        void *h = dlopen(blas, RTLD_NOW);
        if (h) {
            auto setn = (void (*)(int))dlsym(h, "scipy_openblas_set_num_threads");
            if (setn) setn(1);
            or_set_blas((or_sgemm_fn)dlsym(h, "scipy_cblas_sgemm"), (or_dgemm_fn)dlsym(h, "scipy_cblas_dgemm"));
        }
    }
    GTP::setup_default_parameters();
    cfg_num_threads = threads;
    cfg_allow_pondering = false;
    cfg_allow_book = false;
    cfg_quiet = true;
    thread_pool.initialize(cfg_num_threads);
    std::unique_ptr<Random> rng(new Random(5489));
    Zobrist::init_zobrist(*rng);
    Network::get_Network();

    GameState game;
    game.init_game(19, 7.5f);
    for (const char *mv : {"d4", "q16", "q4", "d16", "c14", "r6"}) game.play_textmove(game.get_to_move() ? "w" : "b", mv);

    // one synchronous policy and value evaluation through the backend
    auto direct = Network::get_scored_moves(&game, Network::DIRECT, 0);
    float sum = 0.0f;
    for (auto &sn : direct) sum += sn.first;
    const float v = Network::get_value(&game, Network::DIRECT);

    UCTSearch search(game);
    search.set_playout_limit(playouts);
    search.set_quiet(true);
    const int move = search.think(game.get_to_move());
    opencl.join_outstanding_cb();
    std::printf("RESULT move=%s legal=%d direct_moves=%zu direct_sum=%.6f value=%.6f submitted=%lld sync=%lld "
                "outstanding=%d thread_outstanding=%d\n",
                game.move_to_text(move).c_str(), move == FastBoard::PASS || game.board.get_square(move) == FastBoard::EMPTY,
                direct.size(), sum, v, fake_lg_submitted(), fake_lg_sync_calls(), opencl.m_cb_outstanding.load(),
                opencl_thread_data.m_results_outstanding.load());
    return 0;
}

// search_pattern.cpp -- evaluation requests as the engine's search issues
// them, against the C ABI: leaf evaluations per second on one GPU.
//
// The engine's search (UCTSearch::think on N threads) expands a leaf with an
// asynchronous policy request (UCTNode::netscore_children ->
// Network::async_scored_moves, UCTNode.cpp:74-121, Network.cpp:536-587; at
// most 2 outstanding per thread, OpenCL.cpp:453) and scores it with a
// synchronous value evaluation (UCTNode::run_value_net, UCTNode.cpp:316-344).
// This driver runs N threads that issue exactly that pattern -- no tree, no
// board, no host feature gather, so it measures what the evaluation path can
// serve -- on the benchmark nets (5x5 24->128, 11 x 3x3 128->128, 1x1 head,
// ReLU; value FC 361->256->1, tanh) with random weights and random 0/1
// planes.  The value evaluation of a leaf is either
//   direct: lg_value(ctx, planes, 1, ...), a batch of one per call (the
//           context serialises concurrent calls), or
//   server: lg_submit(ctx, LG_NET_VALUE, planes, 1, ...) and a wait for its
//           completion, so that concurrent requests are merged into batches.
// Each net has its own context (as in the engine's backend) and a drain
// thread that polls completions.
//
// Usage: search_pattern <threads> <seconds> <direct|server> <fp32|bf16|fp16|fp8w> [max_batch]
// Prints one JSON line.
#include "leela_gpu.h"

#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <thread>
#include <vector>

namespace {

constexpr int kPlanes = 24, kPts = 361, kInflight = 2;

struct Req {
    std::atomic<int> done{0};
    std::vector<uint8_t> planes = std::vector<uint8_t>(kPlanes * kPts);
    std::vector<float> out = std::vector<float>(kPts);
};

// Benchmark-net weights in lg_net_desc order: per conv W[O][C][k][k] then
// b[O]; value nets then W1[256][361], b1, W2[256], b2.  He-normal scale,
// zero biases.
std::vector<float> make_weights(const lg_net_desc &d, unsigned seed) {
    std::vector<float> w(lg_weight_count(&d), 0.0f);
    std::mt19937 rng(seed);
    size_t off = 0;
    auto fill = [&](size_t n, int fan_in) {
        std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / (float)fan_in));
        for (size_t i = 0; i < n; ++i) w[off + i] = nd(rng);
        off += n;
    };
    auto conv = [&](int c, int o, int k) {
        fill((size_t)o * c * k * k, c * k * k);
        off += (size_t)o;  // bias
    };
    conv(d.c_in, d.width1, 5);
    for (int l = 0; l < d.n3x3; ++l) conv(l == 0 ? d.width1 : d.width, d.width, 3);
    conv(d.width, 1, d.head_k);
    if (d.value_head) {
        fill((size_t)d.fc_hidden * kPts, kPts);
        off += (size_t)d.fc_hidden;
        fill((size_t)d.fc_hidden, d.fc_hidden);
        off += 1;
    }
    if (off != w.size()) {
        std::fprintf(stderr, "search_pattern: weight layout %zu != %zu\n", off, w.size());
        std::exit(2);
    }
    return w;
}

int precision_of(const char *s) {
    if (!std::strcmp(s, "bf16")) return LG_BF16;
    if (!std::strcmp(s, "fp16")) return LG_FP16;
    if (!std::strcmp(s, "fp8w")) return LG_FP8W;
    return LG_FP32;
}

void check(int rc, const char *what) {
    if (rc < 0) {
        std::fprintf(stderr, "search_pattern: %s: %s\n", what, lg_last_error());
        std::exit(1);
    }
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s threads seconds direct|server fp32|bf16|fp16|fp8w [max_batch]\n", argv[0]);
        return 2;
    }
    const int T = std::atoi(argv[1]);
    const double seconds = std::atof(argv[2]);
    const bool server = !std::strcmp(argv[3], "server");
    const int prec = precision_of(argv[4]);
    const int max_batch = argc > 5 ? std::atoi(argv[5]) : 64;

    lg_net_desc pd{24, 128, 128, 11, 1, LG_ACT_RELU, 0, 0, 0, 0, prec, nullptr};
    lg_net_desc vd{24, 128, 128, 11, 1, LG_ACT_RELU, 0, 1, 256, 0, prec, nullptr};
    const std::vector<float> pw = make_weights(pd, 1), vw = make_weights(vd, 2);
    pd.weights = pw.data();
    vd.weights = vw.data();
    lg_ctx *pc = nullptr, *vc = nullptr;
    check(lg_create(&pd, nullptr, 0, max_batch, &pc), "lg_create policy");
    check(lg_create(nullptr, &vd, 0, max_batch, &vc), "lg_create value");

    std::atomic<bool> stop_drain{false};
    std::atomic<long long> policy_done{0};
    auto drain = [&](lg_ctx *c, bool count) {
        void *tags[256];
        while (!stop_drain.load(std::memory_order_acquire)) {
            const int n = lg_poll(c, tags, 256, 2000);
            check(n, "lg_poll");
            for (int i = 0; i < n; ++i) static_cast<Req *>(tags[i])->done.store(1, std::memory_order_release);
            if (count) policy_done.fetch_add(n, std::memory_order_relaxed);
        }
    };
    std::thread dp(drain, pc, true), dv(drain, vc, false);

    std::atomic<bool> stop{false};
    std::atomic<long long> leaves{0};
    std::atomic<int> failed{0};
    auto worker = [&](int t) {
        std::mt19937 rng(1000 + t);
        std::bernoulli_distribution bit(0.1);
        std::vector<Req> pol(kInflight);
        std::vector<bool> busy(kInflight, false);
        Req val;
        long long mine = 0;
        auto wait_for = [&](Req &r) {
            // bounded: 10 s, then the run is reported as failed
            const auto t0 = std::chrono::steady_clock::now();
            while (!r.done.load(std::memory_order_acquire)) {
                std::this_thread::yield();
                if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(10)) {
                    failed.store(1);
                    return false;
                }
            }
            return true;
        };
        while (!stop.load(std::memory_order_relaxed)) {
            // expand: policy requests up to the per-thread limit
            for (int i = 0; i < kInflight; ++i) {
                if (busy[i] && pol[i].done.load(std::memory_order_acquire)) busy[i] = false;
                if (!busy[i]) {
                    for (auto &x : pol[i].planes) x = bit(rng);
                    pol[i].done.store(0, std::memory_order_relaxed);
                    check(lg_submit(pc, LG_NET_POLICY_LOGITS, pol[i].planes.data(), 1, 1.0f, pol[i].out.data(),
                                    &pol[i]),
                          "lg_submit policy");
                    busy[i] = true;
                }
            }
            // score: the leaf's value
            for (auto &x : val.planes) x = bit(rng);
            if (server) {
                val.done.store(0, std::memory_order_relaxed);
                check(lg_submit(vc, LG_NET_VALUE, val.planes.data(), 1, 1.0f, val.out.data(), &val),
                      "lg_submit value");
                if (!wait_for(val)) break;
            } else {
                check(lg_value(vc, val.planes.data(), 1, val.out.data()), "lg_value");
            }
            ++mine;
        }
        for (int i = 0; i < kInflight; ++i)
            if (busy[i] && !wait_for(pol[i])) break;
        leaves.fetch_add(mine);
    };
    std::vector<std::thread> ws;
    const auto t0 = std::chrono::steady_clock::now();
    for (int t = 0; t < T; ++t) ws.emplace_back(worker, t);
    std::this_thread::sleep_for(std::chrono::duration<double>(seconds));
    stop = true;
    for (auto &w : ws) w.join();
    const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    stop_drain = true;
    dp.join();
    dv.join();
    long long kl = 0, pb = 0, vb = 0;
    lg_stats(pc, &kl, &pb);
    lg_stats(vc, &kl, &vb);
    std::printf("{\"threads\": %d, \"mode\": \"%s\", \"precision\": \"%s\", \"max_batch\": %d, \"seconds\": %.3f, "
                "\"leaf_evals_per_s\": %.1f, \"policy_evals_per_s\": %.1f, \"policy_batches\": %lld, "
                "\"value_batches\": %lld, \"failed\": %d}\n",
                T, server ? "server" : "direct", argv[4], max_batch, el, leaves.load() / el, policy_done.load() / el,
                pb, vb, failed.load());
    lg_destroy(pc);
    lg_destroy(vc);
    return failed.load() ? 1 : 0;
}

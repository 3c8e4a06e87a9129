// fake_lg.cpp -- a CPU stand-in for the parts of the C ABI (leela_gpu.h)
// that the engine-side backend (leela_gb300/integration/opencl_gb300.cpp)
// calls, computed by the oracle (oracle/leela_oracle.c).
//
// TEST INFRASTRUCTURE ONLY: linked into the search-integration test binary
// so that the engine's own search can run against the backend on a machine
// without a GPU.  It checks the backend's plumbing (layer recording,
// synchronous and asynchronous requests, callbacks, throttle, join); the
// numbers come from the oracle, not from libleela_gb300.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "leela_gpu.h"
#include "leela_oracle.h"

namespace {
thread_local std::string t_err;
std::atomic<long long> g_submitted{0}, g_sync_calls{0};
}  // namespace

struct lg_ctx {
    or_net net[2];
    std::vector<float> w[2];
    bool present[2] = {false, false};
    struct Req {
        int net;
        const uint8_t *planes;
        int B;
        float *out;
        void *tag;
    };
    std::mutex mu;
    std::condition_variable cv, dcv;
    std::deque<Req> queue;
    std::deque<void *> done;
    bool stop = false;
    std::thread worker;
};

namespace {
or_net to_or(const lg_net_desc *d) {
    or_net n{};
    n.c_in = d->c_in;
    n.width1 = d->width1;
    n.width = d->width;
    n.n3x3 = d->n3x3;
    n.head_k = d->head_k;
    n.act = d->act;
    n.act_head = d->act_head;
    n.value_head = d->value_head;
    n.fc_hidden = d->fc_hidden;
    n.value_map = d->value_map;
    return n;
}

void run(lg_ctx *c, int net, const uint8_t *planes, int B, float *out) {
    const or_net &n = c->net[net];
    for (int b = 0; b < B; ++b)
        or_forward_f32(&n, c->w[net].data(), planes + (size_t)b * n.c_in * 361, out + (size_t)b * (n.value_head ? 1 : 361),
                       nullptr);
}

void worker(lg_ctx *c) {
    for (;;) {
        lg_ctx::Req r;
        {
            std::unique_lock<std::mutex> lk(c->mu);
            c->cv.wait(lk, [&] { return c->stop || !c->queue.empty(); });
            if (c->queue.empty()) return;
            r = c->queue.front();
            c->queue.pop_front();
        }
        run(c, r.net == LG_NET_VALUE ? 1 : 0, r.planes, r.B, r.out);
        {
            std::lock_guard<std::mutex> lk(c->mu);
            c->done.push_back(r.tag);
        }
        c->dcv.notify_all();
    }
}
}  // namespace

extern "C" {

long long fake_lg_submitted() { return g_submitted.load(); }
long long fake_lg_sync_calls() { return g_sync_calls.load(); }

const char *lg_last_error(void) { return t_err.c_str(); }

int lg_create(const lg_net_desc *policy, const lg_net_desc *value, int, int, lg_ctx **out) {
    lg_ctx *c = new lg_ctx();
    const lg_net_desc *d[2] = {policy, value};
    for (int i = 0; i < 2; ++i) {
        if (!d[i]) continue;
        c->net[i] = to_or(d[i]);
        c->w[i].assign(d[i]->weights, d[i]->weights + or_weight_count(&c->net[i]));
        c->present[i] = true;
    }
    c->worker = std::thread(worker, c);
    *out = c;
    return LG_OK;
}

void lg_destroy(lg_ctx *c) {
    {
        std::lock_guard<std::mutex> lk(c->mu);
        c->stop = true;
    }
    c->cv.notify_all();
    c->worker.join();
    delete c;
}

int lg_policy(lg_ctx *c, const uint8_t *planes, int B, float temperature, float *probs, float *logits) {
    ++g_sync_calls;
    std::vector<float> lg((size_t)B * 361);
    run(c, 0, planes, B, lg.data());
    for (int b = 0; b < B; ++b) or_softmax_f32(lg.data() + (size_t)b * 361, 361, temperature, probs + (size_t)b * 361);
    if (logits) std::memcpy(logits, lg.data(), lg.size() * sizeof(float));
    return LG_OK;
}

int lg_value(lg_ctx *c, const uint8_t *planes, int B, float *value) {
    ++g_sync_calls;
    run(c, 1, planes, B, value);
    return LG_OK;
}

int lg_submit(lg_ctx *c, int net, const uint8_t *planes, int B, float, float *out, void *tag) {
    if (net != LG_NET_POLICY_LOGITS && net != LG_NET_VALUE) {
        t_err = "the stand-in serves head outputs and values only";
        return LG_ERR_ARG;
    }
    ++g_submitted;
    {
        std::lock_guard<std::mutex> lk(c->mu);
        c->queue.push_back({net, planes, B, out, tag});
    }
    c->cv.notify_one();
    return LG_OK;
}

int lg_poll(lg_ctx *c, void **tags, int max, int timeout_us) {
    std::unique_lock<std::mutex> lk(c->mu);
    if (c->done.empty() && timeout_us > 0)
        c->dcv.wait_for(lk, std::chrono::microseconds(timeout_us), [&] { return !c->done.empty(); });
    int n = 0;
    while (n < max && !c->done.empty()) {
        tags[n++] = c->done.front();
        c->done.pop_front();
    }
    return n;
}

}  // extern "C"

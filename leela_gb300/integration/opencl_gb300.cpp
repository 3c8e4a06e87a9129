// opencl_gb300.cpp -- the engine's OpenCL backend (OpenCL.h) on the GB300
// evaluation path.
//
// Build the engine in its OpenCL configuration (its config.h defines
// USE_OPENCL), with this file in place of OpenCL.cpp, this directory on the
// include path before any OpenCL SDK (for CL/cl2.hpp), include/ for
// leela_gpu.h, and link libleela_gb300.  No engine source is edited: the
// engine keeps its feature gather, rotations, softmax, Netresult assembly
// and search (Network.cpp, UCTNode.cpp, UCTSearch.cpp); what this file
// replaces is OpenCL.cpp:441-908.
//
//   OpenCL_Network::push_convolve / push_innerproduct (OpenCL.h:66-87)
//       record the layers as the engine hands them over; the first forward
//       of a net creates its context (lg_create) from them.
//   OpenCL_Network::forward (OpenCL.cpp:490-569)
//       without a callback (the value net, and the policy net's synchronous
//       calls): a request to the batching server that the calling thread
//       waits for, so that the value evaluations of all search threads are
//       merged into GPU batches too (head outputs / the FC output, no map:
//       the engine applies (1 + tanh) / 2 itself, Network.cpp:704-705);
//       LEELA_GB300_SYNC=direct makes them blocking lg_policy / lg_value
//       calls of one position instead;
//       with a callback (Network::async_scored_moves, Network.cpp:536-587):
//       lg_submit of the head outputs, and a drain thread per net runs the
//       callback (forward_cb, Network.cpp:484-534: softmax, Netresult,
//       UCTNode::scoring_cb) for each completed request -- the engine's
//       "async" path really is asynchronous here, and requests of all
//       search threads are merged into GPU batches.
//   OpenCL::thread_can_issue / callback_finished / join_outstanding_cb
//   (OpenCL.cpp:446-577)
//       the engine's per-thread throttle (at most LEELA_GB300_INFLIGHT
//       results outstanding, 2 as in the engine by default) and a bounded
//       join (the engine's is an unbounded spin).
//
// Environment: LEELA_GB300_PRECISION = fp32 (default: the drop-in),
// bf16, fp16 or fp8w for nets the tensor-core path covers;
// LEELA_GB300_DEVICE (default 0); LEELA_GB300_MAX_BATCH (default 64);
// LEELA_GB300_SYNC = server (default) or direct.
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "Network.h"
#include "OpenCL.h"
#include "leela_gpu.h"

OpenCL opencl;
OpenCL_Network opencl_policy_net;
OpenCL_Network opencl_value_net;
thread_local ThreadData opencl_thread_data;

namespace {

int env_int(const char *name, int dflt) {
    const char *v = std::getenv(name);
    return v && *v ? std::atoi(v) : dflt;
}

int env_precision() {
    const char *v = std::getenv("LEELA_GB300_PRECISION");
    if (!v || !*v || !std::strcmp(v, "fp32")) return LG_FP32;
    if (!std::strcmp(v, "bf16")) return LG_BF16;
    if (!std::strcmp(v, "fp16")) return LG_FP16;
    if (!std::strcmp(v, "fp8w")) return LG_FP8W;
    throw std::runtime_error(std::string("LEELA_GB300_PRECISION: unknown precision ") + v);
}

// A request to the batching server: the engine's callback and its data (or,
// for a synchronous call, the flag its thread waits on), and the input
// planes, which must live until the request completes.
struct Pending {
    OpenCL_Network::event_callback cb;
    void *data;
    std::vector<uint8_t> planes;
    std::atomic<int> *done = nullptr;
};

bool sync_direct() {
    static const bool direct = [] {
        const char *v = std::getenv("LEELA_GB300_SYNC");
        return v && !std::strcmp(v, "direct");
    }();
    return direct;
}

// One context per engine net, created on the net's first forward, and the
// thread that hands completed asynchronous requests back to the engine.
struct NetState {
    std::once_flag once;
    lg_ctx *ctx = nullptr;
    int c_in = 0;
    bool value = false;
    std::thread drain;
    std::atomic<bool> stop{false};
    std::string error;

    ~NetState() {
        stop = true;
        if (drain.joinable()) drain.join();
        if (ctx) lg_destroy(ctx);
    }
};

NetState g_policy, g_value;

NetState &state_of(const OpenCL_Network *net) { return net == &opencl_value_net ? g_value : g_policy; }

void drain_main(NetState *st) {
    void *tags[64];
    while (!st->stop.load(std::memory_order_acquire)) {
        const int n = lg_poll(st->ctx, tags, 64, 2000);
        if (n < 0) {
            std::fprintf(stderr, "leela_gb300: a batch failed: %s\n", lg_last_error());
            continue;
        }
        for (int i = 0; i < n; ++i) {
            Pending *pd = static_cast<Pending *>(tags[i]);
            if (pd->done) {
                pd->done->store(1, std::memory_order_release);  // a synchronous call: its thread owns pd
            } else {
                pd->cb(nullptr, CL_COMPLETE, pd->data);
                delete pd;
            }
        }
    }
}

}  // namespace

// --------------------------------------------------------------- OpenCL

void OpenCL::initialize() {
    m_init_ok = true;
    std::fprintf(stderr, "leela_gb300: GB300 evaluation path (device %d)\n", env_int("LEELA_GB300_DEVICE", 0));
}

void OpenCL::ensure_thread_initialized() { opencl_thread_data.m_is_initialized = true; }

std::string OpenCL::get_device_name() { return "GB300 (leela_gb300)"; }

bool OpenCL::thread_can_issue() {
    static const int limit = env_int("LEELA_GB300_INFLIGHT", 2);
    return opencl_thread_data.m_results_outstanding.load() < limit;
}

std::atomic<int> *OpenCL::get_thread_results_outstanding() { return &opencl_thread_data.m_results_outstanding; }

void OpenCL::callback_finished() { m_cb_outstanding.fetch_sub(1, std::memory_order_release); }

void OpenCL::join_outstanding_cb() {
    // Bounded: a request that never completes is reported, not waited for
    // forever.
    const auto limit = std::chrono::steady_clock::now() + std::chrono::seconds(env_int("LEELA_GB300_JOIN_S", 60));
    while (m_cb_outstanding.load(std::memory_order_acquire) > 0) {
        if (std::chrono::steady_clock::now() > limit) {
            std::fprintf(stderr, "leela_gb300: %d callbacks still outstanding after the join limit\n",
                         m_cb_outstanding.load());
            return;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

// ------------------------------------------------------- OpenCL_Network

void OpenCL_Network::add_weights(size_t layer, size_t size, const float *weights) {
    if (layer >= m_layers.size()) m_layers.push_back(Layer());
    m_layers.back().weights.push_back(
        cl::Buffer(CL_MEM_COPY_HOST_PTR | CL_MEM_READ_ONLY, size * sizeof(float), const_cast<float *>(weights)));
}

void OpenCL_Network::forward(std::vector<float> &input, std::vector<float> &output, event_callback cb, void *data) {
    NetState &st = state_of(this);
    std::call_once(st.once, [&] {
        // The layers as pushed (Network.cpp:206-233): convolutions (5x5
        // first, 3x3 trunk, the 1-channel head), then for the value net two
        // inner products.
        std::vector<const Layer *> conv, ip;
        for (auto &l : m_layers) (l.is_innerproduct ? ip : conv).push_back(&l);
        if (conv.size() < 2 || (!ip.empty() && ip.size() != 2))
            throw std::runtime_error("leela_gb300: unexpected layer list");
        std::vector<float> w;
        for (auto &l : m_layers)
            for (auto &buf : l.weights) w.insert(w.end(), buf.floats(), buf.floats() + buf.size() / sizeof(float));
        lg_net_desc d{};
        d.c_in = (int)conv[0]->channels;
        d.width1 = (int)conv[0]->outputs;
        d.width = (int)conv[conv.size() > 2 ? 1 : 0]->outputs;
        d.n3x3 = (int)conv.size() - 2;
        d.head_k = (int)conv.back()->filter_size;
        d.act = LG_ACT_ELU;  // after every layer, the head included (OpenCL.cpp:349-377)
        d.act_head = 1;
        d.value_head = ip.empty() ? 0 : 1;
        d.fc_hidden = ip.empty() ? 0 : (int)ip[0]->outputs;
        d.value_map = 2;     // the engine maps the FC output itself
        d.precision = env_precision();
        d.weights = w.data();
        st.c_in = d.c_in;
        st.value = d.value_head != 0;
        const int rc = st.value ? lg_create(nullptr, &d, env_int("LEELA_GB300_DEVICE", 0),
                                            env_int("LEELA_GB300_MAX_BATCH", 64), &st.ctx)
                                : lg_create(&d, nullptr, env_int("LEELA_GB300_DEVICE", 0),
                                            env_int("LEELA_GB300_MAX_BATCH", 64), &st.ctx);
        if (rc != LG_OK) throw std::runtime_error(std::string("leela_gb300: lg_create: ") + lg_last_error());
        st.drain = std::thread(drain_main, &st);
    });

    opencl.ensure_thread_initialized();
    opencl_thread_data.m_results_outstanding.fetch_add(1, std::memory_order_release);
    std::vector<uint8_t> planes((size_t)st.c_in * 361);
    for (size_t i = 0; i < planes.size(); ++i) planes[i] = (uint8_t)input[i];
    opencl.m_cb_outstanding.fetch_add(1, std::memory_order_release);

    if (cb != nullptr && !st.value) {
        Pending *pd = new Pending{cb, data, std::move(planes)};
        const int rc = lg_submit(st.ctx, LG_NET_POLICY_LOGITS, pd->planes.data(), 1, 1.0f, output.data(), pd);
        if (rc != LG_OK) {
            delete pd;
            throw std::runtime_error(std::string("leela_gb300: lg_submit: ") + lg_last_error());
        }
        return;  // the drain thread runs cb
    }
    int rc;
    if (!sync_direct()) {
        // a request like the asynchronous ones; this thread waits for the
        // drain thread.  The server completes every request it accepted (a
        // failed batch too), so the wait ends; past a minute the process
        // stops rather than free a request the server may still write.
        std::atomic<int> done{0};
        Pending pd{nullptr, nullptr, std::move(planes), &done};
        rc = lg_submit(st.ctx, st.value ? LG_NET_VALUE : LG_NET_POLICY_LOGITS, pd.planes.data(), 1, 1.0f,
                       output.data(), &pd);
        if (rc == LG_OK) {
            const auto t0 = std::chrono::steady_clock::now();
            while (!done.load(std::memory_order_acquire)) {
                std::this_thread::yield();
                if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(60)) {
                    std::fprintf(stderr, "leela_gb300: a synchronous request did not complete within 60 s\n");
                    std::abort();
                }
            }
        }
    } else if (st.value) {
        rc = lg_value(st.ctx, planes.data(), 1, output.data());
    } else {
        std::vector<float> probs(361);
        rc = lg_policy(st.ctx, planes.data(), 1, 1.0f, probs.data(), output.data());
    }
    if (rc != LG_OK) throw std::runtime_error(std::string("leela_gb300: forward: ") + lg_last_error());
    if (cb != nullptr) {
        cb(nullptr, CL_COMPLETE, data);
    } else {
        opencl_thread_data.m_results_outstanding.fetch_sub(1, std::memory_order_release);
        opencl.callback_finished();
    }
}

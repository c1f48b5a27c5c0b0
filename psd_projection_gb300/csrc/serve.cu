// serve.cu — the projection request loop: continuous batching of mixed-size
// projections on one GPU.
//
// The reference library has no serving layer (each call blocks, allocates and
// frees its workspace, and uses the legacy default stream).  An ADMM-style
// caller projects a slowly changing iterate again and again; this engine
// keeps everything such a caller needs on the device and overlaps requests:
//
//   * slots — up to max_slots requests in flight, each on its own CUDA
//     stream with its own workspace, Lanczos state and staging matrix, so
//     requests of different sizes run concurrently on the GPU;
//   * admission by HBM budget — a queued request starts when a slot is free
//     and the slot's buffers for its n fit the budget (slots re-size on
//     demand); requests that do not fit wait while smaller ones start; in
//     submission order, or shortest first (smallest n among each key's
//     oldest queued request), which keeps small requests' latency low when
//     large ones saturate the GPU;
//   * per-key order and warm starts — requests with the same key (one ADMM
//     stream) run in submission order, and each starts its Lanczos bound from
//     the previous request's Ritz vector, kept on the device (with
//     warm_max_iter steps instead of max_iter);
//   * CUDA graphs — with use_graphs, the whole projection of a given n on a
//     slot is captured once and replayed (a few launches per request instead
//     of ~100);
//   * small requests first — with priority_n > 0, requests of n <= priority_n
//     run on high-priority streams; the persistent kernels of larger requests
//     are capped at (SMs - reserve_sms) CTAs, so reserve_sms SMs are always
//     free of them (a small request's short kernels start at once instead of
//     waiting for a large product kernel, which holds every SM it was given
//     until it ends, to drain); and larger requests occupy at most
//     (max_slots - reserve_slots) slots, so a small request never waits for
//     a slot behind a wave of large ones.
//
// Every request's result depends only on its input and its key's previous
// request: kernels are deterministic and a slot's buffers are private while
// it runs, so a result is the same alone and in any mix.
#include <algorithm>
#include <chrono>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "internal.h"

namespace psdgb {
size_t composite_ws_bytes(int64_t n, int precision);
}

namespace {

using psdgb::set_error;

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
    uint64_t ticket;
    int64_t key;
    const double* d_in;
    double* d_out;
    int64_t n;
    double submit_s;
};

struct KeyState {
    double* ritz = nullptr;  // the key's last Ritz vector (warm start), n doubles
    int64_t n = 0;
    bool valid = false;
    bool busy = false;
};

struct Slot {
    cudaStream_t stream = nullptr;   // the stream of the current (or last) request: one of the two below
    cudaStream_t streams[2] = {nullptr, nullptr};  // [0] lowest priority, [1] highest
    cudaEvent_t ev_start = nullptr, ev_end = nullptr;
    int64_t cap_n = 0;          // buffers sized for this n
    size_t bytes = 0;           // device bytes held
    void* buf = nullptr;        // one allocation: matrix | warm | ritz | workspace | lanczos
    double* mat = nullptr;
    double* warm = nullptr;
    double* ritz = nullptr;
    void* ws = nullptr;
    size_t ws_bytes = 0;
    void* lz = nullptr;
    size_t lz_bytes = 0;
    bool busy = false;
    Request req{};
    double start_s = 0.0;
    std::map<std::pair<int64_t, int>, cudaGraphExec_t> graphs;  // (n, warm) -> replayable projection
};

inline size_t up256(size_t x) { return (x + 255) / 256 * 256; }

}  // namespace

struct psdgb_server {
    psdgb_server_config cfg{};
    std::vector<std::unique_ptr<Slot>> slots;
    std::deque<Request> queue;
    std::map<int64_t, KeyState> keys;
    size_t used_bytes = 0;
    uint64_t next_ticket = 1;
    uint64_t completed = 0;
};

namespace {

size_t slot_bytes(const psdgb_server_config& c, int64_t n) {
    const size_t mat = up256(sizeof(double) * n * n);
    const size_t vec = up256(sizeof(double) * n);
    const int64_t iters = c.max_iter > c.warm_max_iter ? c.max_iter : c.warm_max_iter;
    return mat + 2 * vec + up256(psdgb::composite_ws_bytes(n, c.precision)) +
           up256(psdgb::lanczos_state_bytes(n, iters));
}

// Slot buffers come from the stream-ordered allocator on the slot's own
// stream, so re-sizing one slot never synchronises the device while the
// others run.
void slot_release(psdgb_server* s, Slot& sl) {
    for (auto& kv : sl.graphs) cudaGraphExecDestroy(kv.second);
    sl.graphs.clear();
    if (sl.buf) {
        cudaFreeAsync(sl.buf, sl.stream);
        s->used_bytes -= sl.bytes;
    }
    sl.buf = nullptr;
    sl.bytes = 0;
    sl.cap_n = 0;
}

psdgb_status slot_resize(psdgb_server* s, Slot& sl, int64_t n) {
    const psdgb_server_config& c = s->cfg;
    slot_release(s, sl);
    const size_t bytes = slot_bytes(c, n);
    cudaError_t e = cudaMallocAsync(&sl.buf, bytes, sl.stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        sl.buf = nullptr;
        return psdgb::cuda_fail(e, "server slot allocation");
    }
    s->used_bytes += bytes;
    sl.bytes = bytes;
    sl.cap_n = n;
    char* p = static_cast<char*>(sl.buf);
    sl.mat = reinterpret_cast<double*>(p);
    p += up256(sizeof(double) * n * n);
    sl.warm = reinterpret_cast<double*>(p);
    p += up256(sizeof(double) * n);
    sl.ritz = reinterpret_cast<double*>(p);
    p += up256(sizeof(double) * n);
    sl.ws = p;
    sl.ws_bytes = psdgb::composite_ws_bytes(n, c.precision);
    p += up256(sl.ws_bytes);
    sl.lz = p;
    const int64_t iters = c.max_iter > c.warm_max_iter ? c.max_iter : c.warm_max_iter;
    sl.lz_bytes = psdgb::lanczos_state_bytes(n, iters);
    return PSDGB_OK;
}

// The projection of slot.mat (n) with or without the warm start, enqueued on the slot stream.
psdgb_status enqueue_projection(psdgb_server* s, Slot& sl, int64_t n, bool warm) {
    const psdgb_server_config& c = s->cfg;
    return psdgb_composite_auto_scale_async(c.precision, c.schedule, sl.mat, n, warm ? c.warm_max_iter : c.max_iter,
                                            1e-10, 0x5eed5eedull, PSDGB_RESIDUAL_REFERENCE,
                                            warm ? sl.warm : nullptr, sl.ritz, sl.ws, sl.ws_bytes, sl.lz,
                                            sl.lz_bytes, sl.stream);
}

// Small requests (n <= priority_n) go to the slot's high-priority stream;
// large ones to its low-priority stream with their persistent kernels capped.
bool is_small(const psdgb_server_config& c, int64_t n) { return c.priority_n > 0 && n <= c.priority_n; }

struct SmCapScope {  // caps this thread's persistent kernels while a large request is enqueued
    int old;
    explicit SmCapScope(int cap) : old(psdgb::g_sm_cap) { psdgb::g_sm_cap = cap; }
    ~SmCapScope() { psdgb::g_sm_cap = old; }
};

int large_request_cap(const psdgb_server_config& c) {
    if (c.priority_n <= 0 || c.reserve_sms <= 0) return 0;
    psdgb::DeviceState* ds = nullptr;
    if (psdgb::device_state(&ds) != PSDGB_OK) return 0;
    const int cap = ds->sm_count - c.reserve_sms;
    return cap >= 2 ? cap : 2;
}

psdgb_status launch_request(psdgb_server* s, Slot& sl, const Request& r) {
    KeyState& ks = s->keys[r.key];
    const int64_t n = r.n;
    const bool warm = ks.valid && ks.n == n;
    const bool small = is_small(s->cfg, n);
    sl.stream = sl.streams[small ? 1 : 0];
    SmCapScope cap(small ? 0 : large_request_cap(s->cfg));
    PSDGB_CUDA_TRY(cudaEventRecord(sl.ev_start, sl.stream));
    PSDGB_CUDA_TRY(cudaMemcpyAsync(sl.mat, r.d_in, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, sl.stream));
    if (warm) PSDGB_CUDA_TRY(cudaMemcpyAsync(sl.warm, ks.ritz, sizeof(double) * n, cudaMemcpyDeviceToDevice, sl.stream));
    if (s->cfg.use_graphs) {
        auto key = std::make_pair(n, warm ? 1 : 0);
        auto it = sl.graphs.find(key);
        if (it == sl.graphs.end()) {
            cudaGraph_t g = nullptr;
            PSDGB_CUDA_TRY(cudaStreamBeginCapture(sl.stream, cudaStreamCaptureModeThreadLocal));
            psdgb_status st = enqueue_projection(s, sl, n, warm);
            cudaError_t e = cudaStreamEndCapture(sl.stream, &g);
            if (st != PSDGB_OK) {
                if (g) cudaGraphDestroy(g);
                return st;
            }
            if (e != cudaSuccess) return psdgb::cuda_fail(e, "cudaStreamEndCapture");
            cudaGraphExec_t ex = nullptr;
            e = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return psdgb::cuda_fail(e, "cudaGraphInstantiate");
            it = sl.graphs.emplace(key, ex).first;
        }
        PSDGB_CUDA_TRY(cudaGraphLaunch(it->second, sl.stream));
    } else {
        PSDGB_TRY(enqueue_projection(s, sl, n, warm));
    }
    // Keep the key's Ritz vector for its next request; hand out the result.
    if (ks.n != n || ks.ritz == nullptr) {
        if (ks.ritz) {
            cudaFreeAsync(ks.ritz, sl.stream);
            s->used_bytes -= up256(sizeof(double) * ks.n);
        }
        PSDGB_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&ks.ritz), sizeof(double) * n, sl.stream));
        s->used_bytes += up256(sizeof(double) * n);
        ks.n = n;
    }
    PSDGB_CUDA_TRY(cudaMemcpyAsync(ks.ritz, sl.ritz, sizeof(double) * n, cudaMemcpyDeviceToDevice, sl.stream));
    PSDGB_CUDA_TRY(cudaMemcpyAsync(r.d_out, sl.mat, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, sl.stream));
    PSDGB_CUDA_TRY(cudaEventRecord(sl.ev_end, sl.stream));
    ks.valid = true;
    ks.busy = true;
    sl.busy = true;
    sl.req = r;
    sl.start_s = now_s();
    return PSDGB_OK;
}

// Start request r on a free slot whose buffers fit (the smallest such), else
// on a free slot re-sized for it when the budget allows.  *started says
// whether it started; *no_slot that every slot is busy.
psdgb_status try_start(psdgb_server* s, const Request& r, bool* started, bool* no_slot) {
    *started = false;
    *no_slot = false;
    if (s->cfg.priority_n > 0 && s->cfg.reserve_slots > 0 && !is_small(s->cfg, r.n)) {
        int large = 0;
        for (auto& sl : s->slots)
            if (sl->busy && !is_small(s->cfg, sl->req.n)) ++large;
        if (large >= s->cfg.max_slots - s->cfg.reserve_slots) return PSDGB_OK;  // not yet: slots kept for small ones
    }
    Slot* pick = nullptr;
    for (auto& sl : s->slots)
        if (!sl->busy && sl->cap_n >= r.n && (!pick || sl->cap_n < pick->cap_n)) pick = sl.get();
    if (!pick) {
        Slot* spare = nullptr;
        for (auto& sl : s->slots)
            if (!sl->busy && (!spare || sl->bytes < spare->bytes)) spare = sl.get();
        if (!spare) {
            *no_slot = true;
            return PSDGB_OK;
        }
        const size_t need = slot_bytes(s->cfg, r.n) + up256(sizeof(double) * r.n);
        if (s->used_bytes - spare->bytes + need > s->cfg.hbm_budget_bytes) return PSDGB_OK;  // not yet
        // Re-size on the stream the request will run on (stream-ordered allocation).
        spare->stream = spare->streams[is_small(s->cfg, r.n) ? 1 : 0];
        PSDGB_TRY(slot_resize(s, *spare, r.n));
        pick = spare;
    }
    PSDGB_TRY(launch_request(s, *pick, r));
    *started = true;
    return PSDGB_OK;
}

// Start queued requests while slots and budget allow.  FIFO: in submission
// order, skipping requests whose key is in flight or whose buffers do not fit
// yet (a later request of a skipped key never overtakes it).  Shortest first:
// each key's oldest queued request is a candidate (so keys stay in order), and
// candidates start by increasing n, ties by submission.
psdgb_status admit(psdgb_server* s) {
    if (s->cfg.admission == PSDGB_ADMIT_SHORTEST_FIRST) {
        std::map<int64_t, size_t> first;  // key -> queue index of its oldest request
        for (size_t i = 0; i < s->queue.size(); ++i)
            if (!first.count(s->queue[i].key)) first[s->queue[i].key] = i;
        std::vector<size_t> cand;
        for (const auto& kv : first)
            if (!s->keys[kv.first].busy) cand.push_back(kv.second);
        std::sort(cand.begin(), cand.end(), [&](size_t a, size_t b) {
            const Request &ra = s->queue[a], &rb = s->queue[b];
            return ra.n != rb.n ? ra.n < rb.n : ra.ticket < rb.ticket;
        });
        std::vector<uint64_t> done;
        for (size_t i : cand) {
            bool started = false, no_slot = false;
            PSDGB_TRY(try_start(s, s->queue[i], &started, &no_slot));
            if (no_slot) break;
            if (started) done.push_back(s->queue[i].ticket);
        }
        for (uint64_t tk : done)
            for (auto it = s->queue.begin(); it != s->queue.end(); ++it)
                if (it->ticket == tk) {
                    s->queue.erase(it);
                    break;
                }
        return PSDGB_OK;
    }
    std::map<int64_t, bool> blocked_keys;
    for (auto it = s->queue.begin(); it != s->queue.end();) {
        const Request r = *it;
        if (blocked_keys.count(r.key) || s->keys[r.key].busy) {
            blocked_keys[r.key] = true;
            ++it;
            continue;
        }
        bool started = false, no_slot = false;
        PSDGB_TRY(try_start(s, r, &started, &no_slot));
        if (no_slot) break;  // every slot is busy
        if (!started) {
            blocked_keys[r.key] = true;  // does not fit now; smaller requests may
            ++it;
            continue;
        }
        it = s->queue.erase(it);
    }
    return PSDGB_OK;
}

}  // namespace

extern "C" {

double psdgb_clock_seconds(void) { return now_s(); }

psdgb_status psdgb_server_create(const psdgb_server_config* cfg, psdgb_server** out) {
    if (!cfg || !out || cfg->max_slots <= 0 || cfg->max_slots > 256 || cfg->max_iter < 0 || cfg->warm_max_iter < 0 ||
        cfg->priority_n < 0 || cfg->reserve_sms < 0 || cfg->reserve_slots < 0 || cfg->reserve_slots >= cfg->max_slots ||
        (cfg->admission != PSDGB_ADMIT_FIFO && cfg->admission != PSDGB_ADMIT_SHORTEST_FIRST)) {
        set_error("psdgb_server_create: bad configuration");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    psdgb::PrecisionInfo pi{};
    if (!psdgb::precision_info(cfg->precision, &pi) || cfg->precision == PSDGB_PREC_FP32_SIMT) {
        set_error("psdgb_server_create: the server runs the tensor-core precisions");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    // Initialise the library's per-device state and the product kernels'
    // attributes outside any stream capture: one small synchronous projection.
    {
        double* d = nullptr;
        PSDGB_CUDA_TRY(cudaMalloc(&d, sizeof(double) * 128 * 128));
        PSDGB_CUDA_TRY(cudaMemset(d, 0, sizeof(double) * 128 * 128));
        psdgb_status st = psdgb_composite_auto_scale(cfg->precision, cfg->schedule, d, 128, 4, 1e-10, 1,
                                                     PSDGB_RESIDUAL_REFERENCE, nullptr, 0, nullptr, nullptr);
        cudaFree(d);
        if (st != PSDGB_OK) return st;
    }
    auto s = std::make_unique<psdgb_server>();
    s->cfg = *cfg;
    for (int i = 0; i < cfg->max_slots; ++i) {
        auto sl = std::make_unique<Slot>();
        int least = 0, greatest = 0;
        PSDGB_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        PSDGB_CUDA_TRY(cudaStreamCreateWithPriority(&sl->streams[0], cudaStreamNonBlocking, least));
        PSDGB_CUDA_TRY(cudaStreamCreateWithPriority(&sl->streams[1], cudaStreamNonBlocking, greatest));
        sl->stream = sl->streams[0];
        PSDGB_CUDA_TRY(cudaEventCreate(&sl->ev_start));
        PSDGB_CUDA_TRY(cudaEventCreate(&sl->ev_end));
        s->slots.push_back(std::move(sl));
    }
    *out = s.release();
    return PSDGB_OK;
}

psdgb_status psdgb_server_destroy(psdgb_server* s) {
    if (!s) return PSDGB_OK;
    for (auto& sl : s->slots) {
        cudaStreamSynchronize(sl->streams[0]);
        cudaStreamSynchronize(sl->streams[1]);
        slot_release(s, *sl);
        cudaStreamSynchronize(sl->stream);
        cudaEventDestroy(sl->ev_start);
        cudaEventDestroy(sl->ev_end);
        cudaStreamDestroy(sl->streams[0]);
        cudaStreamDestroy(sl->streams[1]);
    }
    cudaDeviceSynchronize();
    for (auto& kv : s->keys)
        if (kv.second.ritz) cudaFree(kv.second.ritz);
    delete s;
    return PSDGB_OK;
}

psdgb_status psdgb_server_submit(psdgb_server* s, int64_t key, const double* d_in, double* d_out, int64_t n,
                                 uint64_t* ticket) {
    if (!s || !d_in || !d_out || n <= 0) {
        set_error("psdgb_server_submit: bad arguments");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (slot_bytes(s->cfg, n) + up256(sizeof(double) * n) > s->cfg.hbm_budget_bytes) {
        set_error("psdgb_server_submit: one request of this size exceeds the server's HBM budget");
        return PSDGB_ERR_OUT_OF_MEMORY;
    }
    Request r{s->next_ticket++, key, d_in, d_out, n, now_s()};
    s->queue.push_back(r);
    if (ticket) *ticket = r.ticket;
    return admit(s);
}

psdgb_status psdgb_server_poll(psdgb_server* s, int wait, psdgb_completion* out, int cap, int* n_out) {
    if (!s || !n_out) {
        set_error("psdgb_server_poll: bad arguments");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    *n_out = 0;
    for (;;) {
        bool any_busy = false;
        for (auto& slp : s->slots) {
            Slot& sl = *slp;
            if (!sl.busy) continue;
            any_busy = true;
            if (*n_out >= cap) break;
            const cudaError_t q = cudaEventQuery(sl.ev_end);
            if (q == cudaErrorNotReady) continue;
            psdgb_completion c{};
            c.ticket = sl.req.ticket;
            c.key = sl.req.key;
            c.n = sl.req.n;
            c.status = (q == cudaSuccess) ? PSDGB_OK : PSDGB_ERR_CUDA;
            c.submit_s = sl.req.submit_s;
            c.start_s = sl.start_s;
            c.end_s = now_s();
            float ms = 0.f;
            if (q == cudaSuccess) cudaEventElapsedTime(&ms, sl.ev_start, sl.ev_end);
            c.gpu_ms = ms;
            if (q != cudaSuccess) cudaGetLastError();
            if (out) out[*n_out] = c;
            ++*n_out;
            sl.busy = false;
            s->keys[sl.req.key].busy = false;
            ++s->completed;
        }
        PSDGB_TRY(admit(s));
        if (*n_out > 0 || !wait || !any_busy) break;
        // Block briefly on the oldest in-flight request instead of spinning.
        Slot* oldest = nullptr;
        for (auto& sl : s->slots)
            if (sl->busy && (!oldest || sl->start_s < oldest->start_s)) oldest = sl.get();
        if (oldest) cudaEventSynchronize(oldest->ev_end);
    }
    return PSDGB_OK;
}

psdgb_status psdgb_server_stats(psdgb_server* s, int* in_flight, int* queued, size_t* bytes_used,
                                uint64_t* completed) {
    if (!s) return PSDGB_ERR_INVALID_ARGUMENT;
    int f = 0;
    for (auto& sl : s->slots) f += sl->busy ? 1 : 0;
    if (in_flight) *in_flight = f;
    if (queued) *queued = static_cast<int>(s->queue.size());
    if (bytes_used) *bytes_used = s->used_bytes;
    if (completed) *completed = s->completed;
    return PSDGB_OK;
}

}  // extern "C"

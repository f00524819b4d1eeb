// serve.cu -- the serving loop of libkmgpu (km_serve_* in include/kmgpu.h).
//
// One native worker thread per server.  Submitted trajectories wait in a
// queue; for every batch the worker picks a leading request -- the one with
// the fewest frames left, or the oldest once it has waited kMaxWaitMs -- and
// packs the queued requests of the leader's center set, fewest frames left
// first, into the batch (a request longer than the batch continues in later
// ones).  It copies them into a device batch slot, runs the assignment
// against the resident center set and copies the labels back.  kSlots slots
// on their own streams rotate, so the copies of one batch overlap the
// kernels of the others.  A batch holds at most kBatchBytes of frames (about
// 0.3 ms on a 200 GB/s host link), so a short request never queues behind
// more than a few short batches, however long the requests ahead of it are.
// The slots are the only device memory the server holds; together they stay
// within the admission budget.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "km_common.cuh"
#include "km_internal.h"

namespace km {
namespace {

using Clock = std::chrono::steady_clock;

constexpr int64_t kDefaultBudget = int64_t(40) << 30;  // 40 GiB
constexpr int kSlots = 3;
constexpr int64_t kBatchBytes = int64_t(64) << 20;  // frame bytes per batch (default)
constexpr int64_t kMinBatchFrames = 4096;
constexpr double kMaxWaitMs = 25.0;  // a request waiting this long leads the next batch

struct Request {
    int32_t set_id = 0;
    const float *X = nullptr;
    int64_t n = 0;
    int32_t d = 0;
    int32_t *labels = nullptr;
    int64_t next = 0;         // first frame not yet placed in a batch
    int64_t pieces_left = 0;  // pieces launched and not yet finished
    int status = KM_PENDING;
    int error = KM_OK;        // first failure of one of its pieces
    std::string error_msg;
    int64_t batch_frames = 0;
    bool started = false;
    Clock::time_point t_submit, t_start, t_done;
};

struct Piece {
    Request *req;
    int64_t src;  // first frame within the request
    int64_t dst;  // first frame within the batch
    int64_t n;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    float *X = nullptr;
    int32_t *labels = nullptr;
    void *ws = nullptr;
    size_t ws_bytes = 0;
    unsigned long long *copy_ctr = nullptr;  // the host copy kernel's counter pair
    uint32_t *err_host = nullptr;  // page-locked
    std::vector<Piece> pieces;
    int64_t frames = 0;
    int launch_status = KM_OK;
    std::string launch_msg;
    bool busy = false;
};

size_t round256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace
}  // namespace km

struct km_server {
    km_serve_config cfg{};
    std::mutex m;
    std::condition_variable cv_work, cv_done;
    std::deque<uint64_t> queue;  // requests with frames not yet placed, oldest first
    std::unordered_map<uint64_t, km::Request> reqs;
    std::vector<const km_centers *> sets;
    uint64_t next_ticket = 1;
    int sets_version = 0;
    bool stop = false;
    km_serve_stats stats{};
    // owned by the worker thread
    km::Slot slots[km::kSlots];
    int slots_version = -1;
    int64_t cap = 0;
    int32_t d_max = 0;
    std::thread worker;
};

namespace km {
namespace {

void free_slot_memory(km_server *S) {
    for (Slot &sl : S->slots) {
        if (sl.X) cudaFree(sl.X);
        if (sl.labels) cudaFree(sl.labels);
        if (sl.ws) cudaFree(sl.ws);
        if (sl.copy_ctr) cudaFree(sl.copy_ctr);
        sl.X = nullptr;
        sl.labels = nullptr;
        sl.ws = nullptr;
        sl.copy_ctr = nullptr;
        sl.ws_bytes = 0;
    }
    S->cap = 0;
}

// Frames per batch for center sets of d features: kBatchBytes of frames (at
// least kMinBatchFrames), or max_batch_frames when the caller set it.
int64_t batch_frames_for(const km_server *S, int32_t d) {
    if (S->cfg.max_batch_frames > 0) return S->cfg.max_batch_frames;
    return std::max<int64_t>(kMinBatchFrames, kBatchBytes / ((int64_t)d * (int64_t)sizeof(float)));
}

// Sizes the slots for the registered center sets: every slot holds the
// largest batch of any set (frames, labels and assignment workspace), and
// all kSlots slots together fit into the budget.
int size_slots(km_server *S, const std::vector<const km_centers *> &sets) {
    free_slot_memory(S);
    int32_t dmax = 1;
    int64_t want = 1;
    for (const km_centers *h : sets) {
        dmax = std::max(dmax, centers_d(h));
        want = std::max(want, batch_frames_for(S, centers_d(h)));
    }
    auto ws_for = [&](int64_t n) {
        size_t ws = 0;
        for (const km_centers *h : sets) ws = std::max(ws, assign_centers_ws_bytes(n, h));
        return ws;
    };
    auto slot_bytes = [&](int64_t n) {
        return round256((size_t)n * dmax * sizeof(float)) + round256((size_t)n * sizeof(int32_t)) +
               round256(ws_for(n)) + round256(2 * sizeof(unsigned long long));
    };
    const uint64_t budget = (uint64_t)S->cfg.hbm_budget_bytes;
    int64_t hi = std::min<int64_t>(want, (int64_t(1) << 31) - 1);
    if (kSlots * (uint64_t)slot_bytes(1) > budget) {
        set_error("admission budget of %lld bytes holds no batch", (long long)budget);
        return KM_ERR_WORKSPACE;
    }
    int64_t lo = 1;
    while (lo < hi) {
        const int64_t mid = lo + (hi - lo + 1) / 2;
        if (kSlots * (uint64_t)slot_bytes(mid) <= budget)
            lo = mid;
        else
            hi = mid - 1;
    }
    const int64_t cap = lo;
    for (Slot &sl : S->slots) {
        sl.ws_bytes = ws_for(cap);
        KM_CUDA(cudaMalloc(&sl.X, (size_t)cap * dmax * sizeof(float)));
        KM_CUDA(cudaMalloc(&sl.labels, (size_t)cap * sizeof(int32_t)));
        if (sl.ws_bytes) KM_CUDA(cudaMalloc(&sl.ws, sl.ws_bytes));
        KM_CUDA(cudaMalloc(&sl.copy_ctr, 2 * sizeof(unsigned long long)));
        KM_CUDA(cudaMemset(sl.copy_ctr, 0, 2 * sizeof(unsigned long long)));
    }
    S->cap = cap;
    S->d_max = dmax;
    std::lock_guard<std::mutex> lk(S->m);
    S->stats.batch_cap_frames = cap;
    S->stats.device_bytes = (int64_t)(kSlots * slot_bytes(cap));
    return KM_OK;
}

// Copies in, assigns and copies out one packed batch; records sl.done.
void launch(km_server *S, Slot &sl, const km_centers *h) {
    cudaStream_t s = sl.stream;
    const int d = centers_d(h);
    int st = KM_OK;
    // Frames into the slot: by a copy kernel where the device reads host
    // memory in place (steadier than the copy engines' reads of page-locked
    // memory, and any host memory works), else by the copy engines.
    const bool in_place = gpu_reads_host_in_place();
    for (const Piece &pc : sl.pieces) {
        if (in_place) {
            st = launch_host_copy(pc.req->X + pc.src * d, sl.X + pc.dst * d, pc.n * d, sl.copy_ctr, s);
            if (st != KM_OK) break;
            continue;
        }
        cudaError_t e = cudaMemcpyAsync(sl.X + pc.dst * d, pc.req->X + pc.src * d, (size_t)pc.n * d * sizeof(float),
                                        cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) {
            st = cuda_fail(e, "cudaMemcpyAsync (frames to the batch slot)");
            break;
        }
    }
    if (st == KM_OK) st = assign_centers_enqueue(sl.X, sl.frames, h, sl.labels, sl.ws, sl.ws_bytes, sl.err_host, s);
    if (st == KM_OK) {
        for (const Piece &pc : sl.pieces) {
            cudaError_t e = cudaMemcpyAsync(pc.req->labels + pc.src, sl.labels + pc.dst, (size_t)pc.n * sizeof(int32_t),
                                            cudaMemcpyDeviceToHost, s);
            if (e != cudaSuccess) {
                st = cuda_fail(e, "cudaMemcpyAsync (labels to the host)");
                break;
            }
        }
    }
    cudaEventRecord(sl.done, s);
    sl.launch_status = st;
    sl.launch_msg = st == KM_OK ? std::string() : std::string(km_last_error());
    sl.busy = true;
    (void)S;
}

// Waits for a launched batch and completes the requests it finished.
void finish(km_server *S, Slot &sl) {
    if (!sl.busy) return;
    int st = sl.launch_status;
    std::string msg = sl.launch_msg;
    cudaError_t e = cudaEventSynchronize(sl.done);
    if (st == KM_OK && e != cudaSuccess) st = cuda_fail(e, "batch");
    if (st == KM_OK) st = device_error_status(*sl.err_host);
    if (st != KM_OK && msg.empty()) msg = km_last_error();
    const Clock::time_point now = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->m);
        for (const Piece &pc : sl.pieces) {
            Request &r = *pc.req;
            if (st != KM_OK && r.error == KM_OK) {
                r.error = st;
                r.error_msg = msg;
            }
            if (--r.pieces_left == 0 && r.next == r.n) {
                r.status = r.error;
                r.t_done = now;
                S->stats.requests += 1;
            }
        }
        S->stats.batches += 1;
        S->stats.frames += sl.frames;
    }
    S->cv_done.notify_all();
    sl.pieces.clear();
    sl.frames = 0;
    sl.busy = false;
}

// Fails every queued request (slot sizing failed).
void fail_queue(km_server *S, int st, const std::string &msg) {
    const Clock::time_point now = Clock::now();
    for (uint64_t t : S->queue) {
        Request &r = S->reqs[t];
        r.error = st;
        r.error_msg = msg;
        r.next = r.n;
        if (r.pieces_left == 0) {
            r.status = st;
            r.t_done = now;
        }
    }
    S->queue.clear();
}

void worker_main(km_server *S) {
    cudaSetDevice(S->cfg.device);
    for (Slot &sl : S->slots) {
        cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        cudaMallocHost(&sl.err_host, sizeof(uint32_t));
    }
    int cur = 0;
    auto finish_all = [&]() {  // oldest batch first
        for (int q = 0; q < kSlots; ++q) finish(S, S->slots[(cur + q) % kSlots]);
    };
    for (;;) {
        std::unique_lock<std::mutex> lk(S->m);
        S->cv_work.wait(lk, [S] { return S->stop || !S->queue.empty(); });
        if (S->queue.empty()) break;  // stop requested and nothing left
        if (S->slots_version != S->sets_version) {
            const std::vector<const km_centers *> sets = S->sets;
            const int version = S->sets_version;
            lk.unlock();
            finish_all();
            const int st = size_slots(S, sets);
            const std::string msg = st == KM_OK ? std::string() : std::string(km_last_error());
            lk.lock();
            S->slots_version = version;
            if (st != KM_OK) {
                fail_queue(S, st, msg);
                lk.unlock();
                S->cv_done.notify_all();
                continue;
            }
        }
        Slot &sl = S->slots[cur];
        if (sl.busy) {
            lk.unlock();
            finish(S, sl);
            lk.lock();
        }
        // Pack.  The leader is the queued request with the fewest frames
        // left (ties: the older), unless the oldest has waited kMaxWaitMs;
        // the leader fixes the center set, and the queued requests of that
        // set follow, fewest frames left first, until the batch is full.
        const Clock::time_point now = Clock::now();
        uint64_t lead = S->queue.front();
        if (std::chrono::duration<double, std::milli>(now - S->reqs[lead].t_submit).count() < kMaxWaitMs) {
            int64_t best = -1;
            for (uint64_t t : S->queue) {
                const Request &r = S->reqs[t];
                if (best < 0 || r.n - r.next < best) {
                    best = r.n - r.next;
                    lead = t;
                }
            }
        }
        const int32_t set_id = S->reqs[lead].set_id;
        const km_centers *h = S->sets[set_id];
        const int64_t cap = std::min<int64_t>(S->cap, batch_frames_for(S, centers_d(h)));
        std::vector<uint64_t> order;  // the leader, then the set's other requests by frames left
        order.push_back(lead);
        for (uint64_t t : S->queue)
            if (t != lead && S->reqs[t].set_id == set_id) order.push_back(t);
        std::stable_sort(order.begin() + 1, order.end(), [S](uint64_t a, uint64_t b) {
            const Request &ra = S->reqs[a], &rb = S->reqs[b];
            return ra.n - ra.next < rb.n - rb.next;
        });
        int64_t filled = 0;
        for (uint64_t t : order) {
            if (filled >= cap) break;
            Request &r = S->reqs[t];
            const int64_t take = std::min(r.n - r.next, cap - filled);
            sl.pieces.push_back(Piece{&r, r.next, filled, take});
            r.next += take;
            r.pieces_left += 1;
            filled += take;
            if (!r.started) {
                r.started = true;
                r.t_start = now;
            }
            if (r.next == r.n) S->queue.erase(std::find(S->queue.begin(), S->queue.end(), t));
        }
        for (const Piece &pc : sl.pieces) pc.req->batch_frames = std::max(pc.req->batch_frames, filled);
        sl.frames = filled;
        lk.unlock();
        launch(S, sl, h);
        cur = (cur + 1) % kSlots;
        bool more;
        {
            std::lock_guard<std::mutex> g(S->m);
            more = !S->queue.empty();
        }
        if (!more) finish_all();  // nothing waiting: deliver what is in flight, oldest first
    }
    finish_all();
    free_slot_memory(S);
    for (Slot &sl : S->slots) {
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.err_host) cudaFreeHost(sl.err_host);
    }
}

}  // namespace
}  // namespace km

using namespace km;

extern "C" {

int km_serve_create(const km_serve_config *config, km_server **out) {
    if (!out) {
        set_error("out must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    *out = nullptr;
    km_serve_config cfg{};
    if (config) cfg = *config;
    if (cfg.hbm_budget_bytes < 0 || cfg.max_batch_frames < 0) {
        set_error("hbm_budget_bytes and max_batch_frames must be >= 0");
        return KM_ERR_BAD_SHAPE;
    }
    if (cfg.hbm_budget_bytes == 0) cfg.hbm_budget_bytes = kDefaultBudget;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (cfg.device < 0 || cfg.device >= ndev) {
        set_error("device %d out of range [0, %d)", cfg.device, ndev);
        return KM_ERR_BAD_SHAPE;
    }
    km_server *S = new km_server();
    S->cfg = cfg;
    S->worker = std::thread(worker_main, S);
    *out = S;
    return KM_OK;
}

int km_serve_add_centers(km_server *S, const km_centers *centers, int32_t *set_id) {
    if (!S || !centers || !set_id) {
        set_error("server, centers and set_id must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    if (centers_device(centers) != S->cfg.device) {
        set_error("center set lives on device %d, the server on device %d", centers_device(centers),
                  S->cfg.device);
        return KM_ERR_BAD_SHAPE;
    }
    std::lock_guard<std::mutex> lk(S->m);
    S->sets.push_back(centers);
    S->sets_version += 1;
    *set_id = (int32_t)S->sets.size() - 1;
    return KM_OK;
}

int km_serve_submit(km_server *S, int32_t set_id, const float *X_host, int64_t n, int32_t d, int32_t *labels_host,
                    uint64_t *ticket) {
    if (!S || !ticket) {
        set_error("server and ticket must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    if (n < 0 || (n > 0 && (!X_host || !labels_host))) {
        set_error("n must be >= 0 with non-NULL X_host and labels_host");
        return KM_ERR_BAD_SHAPE;
    }
    std::unique_lock<std::mutex> lk(S->m);
    if (S->stop) {
        set_error("the server is shutting down");
        return KM_ERR_BAD_SHAPE;
    }
    if (set_id < 0 || set_id >= (int32_t)S->sets.size()) {
        set_error("unknown center set %d", set_id);
        return KM_ERR_BAD_SHAPE;
    }
    if (d != centers_d(S->sets[set_id])) {
        set_error("frames have d=%d, center set %d has d=%d", d, set_id, centers_d(S->sets[set_id]));
        return KM_ERR_BAD_SHAPE;
    }
    const uint64_t t = S->next_ticket++;
    Request &r = S->reqs[t];
    r.set_id = set_id;
    r.X = X_host;
    r.n = n;
    r.d = d;
    r.labels = labels_host;
    r.t_submit = Clock::now();
    if (n == 0) {
        r.status = KM_OK;
        r.t_start = r.t_done = r.t_submit;
        S->stats.requests += 1;
    } else {
        S->queue.push_back(t);
    }
    *ticket = t;
    lk.unlock();
    S->cv_work.notify_one();
    return KM_OK;
}

int km_serve_poll(km_server *S, uint64_t ticket, int32_t timeout_ms, km_request_info *info) {
    if (!S) {
        set_error("server must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    std::unique_lock<std::mutex> lk(S->m);
    // Look the ticket up again after every wake-up: submissions from other
    // threads may rehash the table while this thread waits.
    auto done = [&] {
        auto f = S->reqs.find(ticket);
        return f == S->reqs.end() || f->second.status != KM_PENDING;
    };
    if (timeout_ms < 0)
        S->cv_done.wait(lk, done);
    else
        S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end()) {
        set_error("unknown ticket %llu", (unsigned long long)ticket);
        return KM_ERR_BAD_SHAPE;
    }
    const Request &r = it->second;
    if (info) {
        std::memset(info, 0, sizeof(*info));
        info->status = r.status;
        info->set_id = r.set_id;
        info->n_frames = r.n;
        info->batch_frames = r.batch_frames;
        if (r.started) info->queue_ms = std::chrono::duration<double, std::milli>(r.t_start - r.t_submit).count();
        if (r.status != KM_PENDING)
            info->total_ms = std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count();
    }
    const int st = r.status;
    if (st == KM_PENDING) return KM_PENDING;
    if (st != KM_OK) set_error("%s", r.error_msg.c_str());
    S->reqs.erase(it);
    return st;
}

int km_serve_stats_read(km_server *S, km_serve_stats *stats) {
    if (!S || !stats) {
        set_error("server and stats must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    std::lock_guard<std::mutex> lk(S->m);
    *stats = S->stats;
    return KM_OK;
}

int km_serve_shutdown(km_server *S) {
    if (!S) return KM_OK;
    {
        std::lock_guard<std::mutex> lk(S->m);
        S->stop = true;
    }
    S->cv_work.notify_all();
    if (S->worker.joinable()) S->worker.join();
    delete S;
    return KM_OK;
}

}  // extern "C"

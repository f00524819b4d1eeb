// capi.cu -- the extern "C" entry points of libkmgpu (declared in
// include/kmgpu.h).  Each one validates its arguments, carves the caller's
// workspace and enqueues kernels on the caller's stream.
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "km_common.cuh"
#include "km_internal.h"

namespace km {

namespace {
thread_local char g_last_error[512] = "";
}

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

namespace {
struct ProfTotals {
    std::mutex m;
    bool on = false;
    double ms[kProfKinds] = {};
    int64_t n[kProfKinds] = {};
} g_prof;
}  // namespace

int ProfEvents::open() {
    {
        std::lock_guard<std::mutex> lk(g_prof.m);
        active = g_prof.on;
    }
    if (!active) return KM_OK;
    for (int i = 0; i < kProfKinds; ++i)
        for (int j = 0; j < 2; ++j) KM_CUDA(cudaEventCreate(&ev[i][j]));
    return KM_OK;
}

void ProfEvents::close() {
    for (int i = 0; i < kProfKinds; ++i)
        for (int j = 0; j < 2; ++j)
            if (ev[i][j]) {
                cudaEventDestroy(ev[i][j]);
                ev[i][j] = nullptr;
            }
    active = false;
}

// While a stream is being captured, cudaEventRecordExternal makes the record
// an event-record node of the graph (a plain record would only be a capture
// dependency); outside capture the flag is not allowed.
static void record_event(cudaEvent_t ev, cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &st) == cudaSuccess && st == cudaStreamCaptureStatusActive)
        cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal);
    else
        cudaEventRecord(ev, s);
}

void ProfEvents::begin(int kind, cudaStream_t s) {
    if (!active) return;
    record_event(ev[kind][0], s);
    used[kind] = true;
}

void ProfEvents::end(int kind, cudaStream_t s) {
    if (active) record_event(ev[kind][1], s);
}

void ProfEvents::collect() {
    if (!active) return;
    std::lock_guard<std::mutex> lk(g_prof.m);
    for (int i = 0; i < kProfKinds; ++i) {
        if (!used[i]) continue;
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, ev[i][0], ev[i][1]) == cudaSuccess) {
            g_prof.ms[i] += ms;
            g_prof.n[i] += 1;
        } else {
            cudaGetLastError();  // a failed read must not surface at the next launch check
        }
    }
}

namespace {

// The tensor-core precisions (FP16, BF16 or FP8 operands, exact re-check).
inline bool is_tc(int prec) { return prec == KM_PREC_FP16 || prec == KM_PREC_BF16 || prec == KM_PREC_FP8; }

// Precisions chosen by km_tune, per (d, k).
struct TuneCache {
    std::mutex m;
    std::map<std::pair<int, int>, int> choice;
} g_tune;

// KM_PREC_AUTO: a km_tune result for (d, k) if there is one, else the rule
// measured on the precision sweep (1M frames, d 16..1024, k 100..5000): the
// tensor-core path wins from d >= 64 at every k, and for d >= 16 once
// k >= 1000; below that the exact FP32 kernel is as fast or faster.
int resolve_precision(int precision, int d, int k, bool check_device) {
    if (precision != KM_PREC_AUTO) return precision;
    {
        std::lock_guard<std::mutex> lk(g_tune.m);
        auto it = g_tune.choice.find(std::make_pair(d, k));
        if (it != g_tune.choice.end()) return it->second;
    }
    const bool tc_ok = check_device ? tc_supported(d, k) : tc_plan_exists(d, k);
    // Measured on GB300 (1-4.3M frames): FP16 + re-check wins from d = 64 at
    // every k, and from d = 8 once k >= 1000 (d = 10, k = 1000: 2.5 against
    // 7.2 ms per Lloyd iteration; d = 16, k = 1000: 1.4 against 2.7 ms).
    if (tc_ok && (d >= 64 || (d >= 8 && k >= 1000))) return KM_PREC_FP16;
    return KM_PREC_FP32;
}

struct AssignWs {
    TcBuffers tc;
};

size_t assign_ws_bytes(int64_t n, int d, int k, int prec) {
    if (!is_tc(prec)) return 0;
    return tc_frames_ws_size(n, d) + tc_centers_ws_size(d, k) + tc_assign_ws_size(n, d, k) + 3 * 256;
}

void carve_assign(void *ws, int64_t n, int d, int k, TcBuffers &b) {
    char *p = static_cast<char *>(ws);
    tc_carve_frames(p, n, d, b);
    p += (tc_frames_ws_size(n, d) + 255) / 256 * 256;
    tc_carve_centers(p, d, k, b);
    p += (tc_centers_ws_size(d, k) + 255) / 256 * 256;
    tc_carve_assign(p, n, d, k, b);
}

int check_device_errors(uint32_t e) {
    if (e & kDevBadLabel) {
        set_error("a label is outside [0, k)");
        return KM_ERR_BAD_LABEL;
    }
    if (e & (kDevTimeoutTma | kDevTimeoutMma | kDevTimeoutEpi)) {
        set_error("a device-side wait expired (error word 0x%x)", e);
        return KM_ERR_TIMEOUT;
    }
    return KM_OK;
}

// The assignment once the precision is resolved and the workspace checked.
// For the tensor-core precisions, b holds the carved buffers (operand type set);
// centers_ready means the
// center half (FP16 copy, norms, shift, scale) is already prepared.
int assign_core(const float *X, int64_t n, int32_t d, const float *C, int32_t k, int prec, int32_t *labels,
                TcBuffers &b, bool centers_ready, km_assign_stats *stats, cudaStream_t s,
                const PairSrc *ps = nullptr) {
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->n_frames = n;
        stats->precision = prec;
    }
    if (n == 0) return KM_OK;
    ProfEvents prof;
    KM_TRY(prof.open());
    struct Closer {
        ProfEvents &p;
        ~Closer() { p.close(); }
    } closer{prof};
    if (prec == KM_PREC_FP32) {
        prof.begin(kProfFp32, s);
        KM_TRY(launch_assign_fp32(X, nullptr, nullptr, n, d, C, k, labels, nullptr, nullptr, s, ps));
        prof.end(kProfFp32, s);
        if (stats || prof.active) KM_CUDA(cudaStreamSynchronize(s));
        prof.collect();
        return KM_OK;
    }
    if (!centers_ready) {
        KM_TRY(tc_prepare_shift_from_centers(C, d, k, b, s));
        KM_TRY(tc_prepare_centers(C, d, k, b, s));
    }
    KM_TRY(tc_prepare_frames(X, n, d, b, s, ps));
    KM_TRY(tc_assign(X, n, d, C, k, labels, b, s, &prof, nullptr, nullptr, ps));
    if (prof.active) {
        KM_CUDA(cudaStreamSynchronize(s));
        prof.collect();
    }
    if (stats) {
        int32_t cnt[3];
        unsigned long long flips = 0;
        uint32_t err = 0;
        KM_CUDA(cudaMemcpyAsync(cnt, b.counters, sizeof(cnt), cudaMemcpyDeviceToHost, s));
        KM_CUDA(cudaMemcpyAsync(&flips, b.flipped, sizeof(flips), cudaMemcpyDeviceToHost, s));
        KM_CUDA(cudaMemcpyAsync(&err, b.err, sizeof(err), cudaMemcpyDeviceToHost, s));
        KM_CUDA(cudaStreamSynchronize(s));
        stats->n_recheck = cnt[0];
        stats->n_full = cnt[1];
        stats->n_pairs = cnt[2];
        stats->n_flipped = (int64_t)flips;
        KM_TRY(check_device_errors(err));
    }
    return KM_OK;
}

int assign_impl(const float *X, int64_t n, int32_t d, const float *C, int32_t k, int32_t precision,
                int32_t *labels, void *ws, size_t ws_bytes, km_assign_stats *stats, cudaStream_t s,
                const PairSrc *ps = nullptr) {
    KM_TRY(check_shape(n, d, k));
    if ((n > 0 && ((!X && !ps) || !labels)) || !C) {
        set_error("X, C and labels must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    int prec = resolve_precision(precision, d, k, true);
    if (prec != KM_PREC_FP32 && !is_tc(prec)) {
        set_error("unknown precision %d", precision);
        return KM_ERR_BAD_SHAPE;
    }
    if (is_tc(prec) && !tc_supported(d, k)) {
        set_error("no tensor-core kernel for d=%d, k=%d on this device", d, k);
        return KM_ERR_UNSUPPORTED;
    }
    KM_TRY(check_ws(ws, ws_bytes, assign_ws_bytes(n, d, k, prec)));
    TcBuffers b;
    if (is_tc(prec) && n > 0) {
        carve_assign(ws, n, d, k, b);
        tc_set_operand(b, d, prec);
    }
    if (ps && prec == KM_PREC_FP8) {
        set_error("FP8 operands are not built for coordinate frames");
        return KM_ERR_UNSUPPORTED;
    }
    return assign_core(X, n, d, C, k, prec, labels, b, false, stats, s, ps);
}

// Workspace of an assignment whose centers are prepared: frames + lists.
size_t resident_ws_bytes(int64_t n, int d, int k, int prec) {
    if (!is_tc(prec)) return 0;
    return tc_frames_ws_size(n, d) + tc_assign_ws_size(n, d, k) + 2 * 256;
}

// dst (device) <- src (host memory that the device reads in place, or any
// device-visible memory), count floats.  The CTAs claim blocks of
// kCopyBlock floats in order from ctr[0], so a CTA that is placed late
// (behind the CTAs of a kernel that fills the SM's registers or threads)
// takes fewer blocks instead of holding back the end of the copy; each CTA
// asks for its next block while it copies the current one.  The CTA that
// finishes last sets the counter pair ctr = {next block, CTAs done} back to
// zero for the next launch on the stream (it is zero before the first).
// One CTA of 128 threads per SM with at most 32 registers a thread fits
// beside a tensor-core CTA and beside the re-check's CTAs; 16-byte words
// where both ends are aligned, else 4-byte words.
constexpr int kCopyThreads = 128;
constexpr int64_t kCopyBlock = 4096;  // floats per claimed block (16 KB)

__global__ void __launch_bounds__(kCopyThreads, 16) host_copy_kernel(const float *__restrict__ src,
                                                                     float *__restrict__ dst, int64_t count,
                                                                     unsigned long long *__restrict__ ctr) {
    __shared__ unsigned long long claim[2];
    const unsigned long long nblk = (unsigned long long)((count + kCopyBlock - 1) / kCopyBlock);
    const bool vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0;
    if (threadIdx.x == 0) claim[0] = atomicAdd(ctr, 1ull);
    __syncthreads();
    int cur = 0;
    for (;;) {
        const unsigned long long b = claim[cur];
        if (b >= nblk) break;  // the same value in every thread
        const int64_t a = (int64_t)b * kCopyBlock;
        const int64_t e = count - a < kCopyBlock ? count : a + kCopyBlock;
        if (vec && e - a == kCopyBlock) {
            // 1024 float4 words: two rounds of four per thread
            const float4 *s4 = reinterpret_cast<const float4 *>(src + a);
            float4 *d4 = reinterpret_cast<float4 *>(dst + a);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                float4 v[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) v[q] = s4[(h * 4 + q) * kCopyThreads + threadIdx.x];
                if (h == 0 && threadIdx.x == 0) claim[cur ^ 1] = atomicAdd(ctr, 1ull);
#pragma unroll
                for (int q = 0; q < 4; ++q) d4[(h * 4 + q) * kCopyThreads + threadIdx.x] = v[q];
            }
        } else {
            if (threadIdx.x == 0) claim[cur ^ 1] = atomicAdd(ctr, 1ull);
            for (int64_t i = a + threadIdx.x; i < e; i += kCopyThreads) dst[i] = src[i];
        }
        __syncthreads();  // the next claim is visible; this one is no longer read
        cur ^= 1;
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(ctr + 1, 1ull) == (unsigned long long)gridDim.x - 1) {
            ctr[0] = 0ull;
            ctr[1] = 0ull;
        }
    }
}

// Graphs keep the launch priority of their kernel nodes (the chunked
// tensor-core pass runs at the greatest priority); without that flag a graph
// runs every node at its stream's priority.
cudaError_t instantiate_with_priorities(cudaGraphExec_t *gx, cudaGraph_t g) {
    cudaError_t e = cudaGraphInstantiate(gx, g, cudaGraphInstantiateFlagUseNodePriority);
    if (e != cudaSuccess) {
        cudaGetLastError();
        e = cudaGraphInstantiate(gx, g, 0);
    }
    return e;
}

// Iterations after the first one can run as a CUDA graph WHILE loop: its
// body is one iteration plus lloyd_loop_step_kernel, which records the
// inertia, applies the stopping rule on the device and sets the loop's
// condition, so a run of iterations costs one launch and one read-back.
// A launch runs at most kLoopBatch iterations (the size of the inertia
// buffer in the workspace).
struct LoopState {
    double prev;
    double tol;
    int32_t it;      // iterations run by this launch
    int32_t max_it;  // bound for this launch
    int32_t converged;
    uint32_t err;
};
constexpr int kLoopBatch = 64;

__global__ void lloyd_loop_step_kernel(LoopState *st, const double *cost, const uint32_t *err_update,
                                       const uint32_t *err_tc, double *inertias, cudaGraphConditionalHandle h) {
    const double c = *cost;
    const uint32_t e = *err_update | (err_tc ? *err_tc : 0u);
    const int it = st->it;
    inertias[it] = c;
    // the host loop's rule: rel = |cost - prev| / cost (0 when cost is 0)
    const double rel = c != 0.0 ? fabs(c - st->prev) / c : 0.0;
    st->prev = c;
    st->it = it + 1;
    st->err |= e;
    const int conv = rel <= st->tol ? 1 : 0;
    st->converged = conv;
    cudaGraphSetConditional(h, (conv || e != 0u || it + 1 >= st->max_it) ? 0u : 1u);
}

size_t lloyd_ws_bytes(int64_t n, int d, int k, int prec) {
    Carver c(nullptr);
    c.take<unsigned long long>(2);  // host copy counter pair
    c.take<LoopState>(1);
    c.take<double>(kLoopBatch);
    c.take<char>(update_ws_size(n, d, k));
    c.take<float>((size_t)k * d);  // C_new
    c.take<double>(1);             // cost
    c.take<uint32_t>(1);           // error word
    c.take<char>(assign_ws_bytes(n, d, k, prec));
    if (is_tc(prec)) {
        c.take<int32_t>(3 * (size_t)n);  // flip list
        c.take<int32_t>(1);              // its count
    }
    return c.bytes();
}

}  // namespace
}  // namespace km

using namespace km;

// A resident center set (include/kmgpu.h).
struct km_centers {
    int32_t k = 0, d = 0, prec = KM_PREC_FP32;
    int device = 0;
    void *mem = nullptr;
    size_t bytes = 0;
    float *C = nullptr;
    TcBuffers tc;  // center half: ch, cnorm, shift, scal (tensor-core precisions)
};

namespace km {
// Enqueues the assignment of n frames against a resident center set without
// synchronising: the device error word (tensor-core waits) is copied to
// err_host (host, ideally pinned) on the same stream, 0 for KM_PREC_FP32.
int assign_centers_enqueue(const float *X, int64_t n, const km_centers *h, int32_t *labels, void *ws,
                           size_t ws_bytes, uint32_t *err_host, cudaStream_t s) {
    *err_host = 0;
    KM_TRY(check_ws(ws, ws_bytes, resident_ws_bytes(n, h->d, h->k, h->prec)));
    if (n == 0) return KM_OK;
    if (h->prec == KM_PREC_FP32)
        return launch_assign_fp32(X, nullptr, nullptr, n, h->d, h->C, h->k, labels, nullptr, nullptr, s);
    TcBuffers b = h->tc;
    char *p = static_cast<char *>(ws);
    tc_carve_frames(p, n, h->d, b);
    p += (tc_frames_ws_size(n, h->d) + 255) / 256 * 256;
    tc_carve_assign(p, n, h->d, h->k, b);
    tc_set_operand(b, h->d, h->prec);
    KM_TRY(tc_prepare_frames(X, n, h->d, b, s));
    KM_TRY(tc_assign(X, n, h->d, h->C, h->k, labels, b, s, nullptr));
    KM_CUDA(cudaMemcpyAsync(err_host, b.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    return KM_OK;
}

size_t assign_centers_ws_bytes(int64_t n, const km_centers *h) { return resident_ws_bytes(n, h->d, h->k, h->prec); }
int centers_d(const km_centers *h) { return h->d; }
int centers_device(const km_centers *h) { return h->device; }
int device_error_status(uint32_t e) { return check_device_errors(e); }

// Test hook: bits that the next km_update / km_update_noalloc call adds to
// the error word it reads back from the device, as if a kernel had set them.
// It lets the tests check how each bit maps to a status without making a
// device-side wait run out.
static std::atomic<uint32_t> g_fake_device_error{0};
uint32_t take_fake_device_error() { return g_fake_device_error.exchange(0u); }
}  // namespace km

extern "C" {

int km_version(void) { return 1; }

const char *km_status_string(int status) {
    switch (status) {
        case KM_OK: return "ok";
        case KM_ERR_BAD_SHAPE: return "bad shape or argument";
        case KM_ERR_WORKSPACE: return "workspace too small";
        case KM_ERR_NON_FINITE: return "non-finite input";
        case KM_ERR_TIMEOUT: return "device wait timed out";
        case KM_ERR_CUDA: return "CUDA error";
        case KM_ERR_UNSUPPORTED: return "unsupported on this device";
        case KM_ERR_BAD_LABEL: return "label out of range";
        default: return "unknown status";
    }
}

const char *km_last_error(void) { return g_last_error; }

int km_debug_fake_device_error(uint32_t bits) {
    g_fake_device_error.store(bits);
    return KM_OK;
}

int km_profile_enable(int on) {
    std::lock_guard<std::mutex> lk(g_prof.m);
    g_prof.on = on != 0;
    for (int i = 0; i < kProfKinds; ++i) {
        g_prof.ms[i] = 0.0;
        g_prof.n[i] = 0;
    }
    return KM_OK;
}

int km_profile_read(int32_t kind, double *ms_total, int64_t *launches) {
    if (kind < 0 || kind >= kProfKinds || !ms_total || !launches) {
        set_error("kind must be in [0, %d) and the outputs non-NULL", (int)kProfKinds);
        return KM_ERR_BAD_SHAPE;
    }
    std::lock_guard<std::mutex> lk(g_prof.m);
    *ms_total = g_prof.ms[kind];
    *launches = g_prof.n[kind];
    return KM_OK;
}

size_t km_assign_workspace_size(int64_t n, int32_t d, int32_t k, int32_t precision) {
    if (check_shape(n, d, k) != KM_OK) return 0;
    return assign_ws_bytes(n, d, k, resolve_precision(precision, d, k, false));
}

int km_assign(const float *X, int64_t n, int32_t d, const float *C, int32_t k, int32_t precision,
              int32_t *labels, void *workspace, size_t workspace_bytes, km_assign_stats *stats,
              void *stream) {
    return assign_impl(X, n, d, C, k, precision, labels, workspace, workspace_bytes, stats,
                       static_cast<cudaStream_t>(stream));
}

int km_batch_assign(const float *X_packed, const int64_t *offsets, int32_t n_traj, int32_t d,
                    const float *C, int32_t k, int32_t precision, int32_t *labels_packed,
                    void *workspace, size_t workspace_bytes, km_assign_stats *stats, void *stream) {
    if (n_traj < 0 || (n_traj > 0 && !offsets)) {
        set_error("n_traj must be >= 0 with n_traj+1 offsets");
        return KM_ERR_BAD_SHAPE;
    }
    if (n_traj > 0 && offsets[0] != 0) {
        set_error("offsets[0] must be 0");
        return KM_ERR_BAD_SHAPE;
    }
    for (int32_t t = 0; t < n_traj; ++t) {
        if (offsets[t + 1] < offsets[t]) {
            set_error("offsets must be non-decreasing (trajectory %d)", t);
            return KM_ERR_BAD_SHAPE;
        }
    }
    const int64_t n = n_traj > 0 ? offsets[n_traj] : 0;
    return assign_impl(X_packed, n, d, C, k, precision, labels_packed, workspace, workspace_bytes, stats,
                       static_cast<cudaStream_t>(stream));
}

int km_debug_tc_distances(const float *X, int64_t n, int32_t d, const float *C, int32_t k, int32_t precision,
                          float *V, int32_t *labels, uint64_t *wait_cycles, void *workspace, size_t workspace_bytes,
                          void *stream) {
    KM_TRY(check_shape(n, d, k));
    if (n > 0 && (!X || !labels || !C)) {
        set_error("X, C and labels must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    if (!is_tc(precision)) {
        set_error("km_debug_tc_distances runs a tensor-core precision (FP16, BF16 or FP8), not %d", precision);
        return KM_ERR_BAD_SHAPE;
    }
    if (!tc_supported(d, k)) {
        set_error("no tensor-core kernel for d=%d, k=%d on this device", d, k);
        return KM_ERR_UNSUPPORTED;
    }
    KM_TRY(check_ws(workspace, workspace_bytes, assign_ws_bytes(n, d, k, KM_PREC_FP16)));
    if (n == 0) return KM_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    TcBuffers b;
    carve_assign(workspace, n, d, k, b);
    tc_set_operand(b, d, precision);
    KM_TRY(tc_prepare_shift_from_centers(C, d, k, b, s));
    KM_TRY(tc_prepare_centers(C, d, k, b, s));
    KM_TRY(tc_prepare_frames(X, n, d, b, s));
    // The 8 wait counters live in the unused tail of the candidate counters block.
    unsigned long long *dev_wait = nullptr;
    if (wait_cycles) {
        dev_wait = reinterpret_cast<unsigned long long *>(b.counters + 4);
        KM_CUDA(cudaMemsetAsync(dev_wait, 0, 8 * sizeof(unsigned long long), s));
    }
    KM_TRY(tc_assign(X, n, d, C, k, labels, b, s, nullptr, V, dev_wait));
    if (wait_cycles)
        KM_CUDA(cudaMemcpyAsync(wait_cycles, dev_wait, 8 * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    KM_CUDA(cudaStreamSynchronize(s));
    return KM_OK;
}

size_t km_update_workspace_size(int64_t n, int32_t d, int32_t k) {
    if (check_shape(n, d, k) != KM_OK) return 0;
    return update_ws_size(n, d, k) + 256;
}

int km_update(const float *X, int64_t n, int32_t d, const int32_t *labels, int32_t k,
              const float *C_old, float *C_new, int64_t *counts, double *cost, void *workspace,
              size_t workspace_bytes, void *stream) {
    KM_TRY(check_shape(n, d, k));
    if ((n > 0 && (!X || !labels)) || !C_old || !C_new || !cost) {
        set_error("X, labels, C_old, C_new and cost must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    if (C_old == C_new) {
        set_error("C_new must not alias C_old");
        return KM_ERR_BAD_SHAPE;
    }
    const size_t need = update_ws_size(n, d, k) + 256;
    KM_TRY(check_ws(workspace, workspace_bytes, need));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t *err = reinterpret_cast<uint32_t *>(static_cast<char *>(workspace) + update_ws_size(n, d, k));
    KM_CUDA(cudaMemsetAsync(err, 0, sizeof(uint32_t), s));
    KM_TRY(launch_update(X, n, d, labels, k, C_old, C_new, counts, cost, err, workspace, s));
    uint32_t e = 0;
    KM_CUDA(cudaMemcpyAsync(&e, err, sizeof(e), cudaMemcpyDeviceToHost, s));
    KM_CUDA(cudaStreamSynchronize(s));
    return check_device_errors(e | take_fake_device_error());
}

size_t km_kmpp_workspace_size(int64_t n, int32_t d, int32_t k) {
    if (check_shape(n, d, k) != KM_OK) return 0;
    return kmpp_ws_size(n, d, k);
}

int km_kmpp(const float *X, int64_t n, int32_t d, int32_t k, uint32_t seed, float *C0, int64_t *idx,
            km_callback cb, void *cb_user, void *workspace, size_t workspace_bytes, void *stream) {
    KM_TRY(check_shape(n, d, k));
    if (n < 1 || !X || !C0) {
        set_error("kmeans++ needs n >= 1 and non-NULL X, C0");
        return KM_ERR_BAD_SHAPE;
    }
    KM_TRY(check_ws(workspace, workspace_bytes, kmpp_ws_size(n, d, k)));
    return run_kmpp(X, n, d, k, seed, C0, idx, cb, cb_user, workspace, static_cast<cudaStream_t>(stream));
}

size_t km_lloyd_workspace_size(int64_t n, int32_t d, int32_t k, int32_t precision) {
    if (check_shape(n, d, k) != KM_OK) return 0;
    return lloyd_ws_bytes(n, d, k, resolve_precision(precision, d, k, false));
}

}  // extern "C"

namespace {

// Host frames of km_lloyd_host: n_parts row-major float32 blocks, copied one
// after the other into the device frame buffer.
struct HostFrames {
    const float *const *parts;
    const int64_t *rows;
    int32_t n_parts;
};

// Rows per streamed chunk of the first iteration: about 1/24 of the run,
// at least 16384 frames, a multiple of 256.  (Halving the last chunks down
// to 16384 frames did not shorten the run: every chunk carries a fixed
// train of small launches.)
int64_t stream_chunk_rows(int64_t n) {
    int64_t c = (n + 23) / 24;
    if (c < 16384) c = 16384;
    return (c + 255) / 256 * 256;
}

// ---------------------------------------------------------------------------
// Staged copies of pageable host frames.  A cudaMemcpyAsync from pageable
// memory is staged by the driver and returns only when the copy is done, so
// the host could not enqueue the first iteration's kernels until every frame
// had crossed the link.  Here worker threads copy blocks of at most
// kStageBytes from the caller's arrays into page-locked buffers (two per
// worker) and issue each block's host-to-device copy on the worker's own
// stream, with an event per block; the enqueue of a chunk's kernels waits on
// the host until the chunk's blocks are issued, then on their events on the
// device.  The page-locked ring is allocated once per process and kept.
// ---------------------------------------------------------------------------
constexpr size_t kStageBytes = size_t(16) << 20;

struct StagePool {
    std::mutex use;  // held by the call that stages (one at a time)
    std::vector<void *> bufs;
    int device = -1;
};
StagePool &stage_pool() {
    static StagePool *p = new StagePool();  // kept until exit: buffers may be in use at static destruction
    return *p;
}

// One worker per host core but one (the calling thread enqueues the
// kernels), at most 16: a single core's memcpy moves far less than the host
// link carries.
int stage_workers() {
    const unsigned hw = std::thread::hardware_concurrency();
    int w = hw ? (int)hw - 1 : 4;
    return std::max(2, std::min(16, w));
}

// True when the host memory at p is ordinary pageable memory.
bool is_pageable(const void *p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return true;
    }
    return a.type == cudaMemoryTypeUnregistered;
}

// True when some part of the host frames is ordinary pageable memory.
bool has_pageable_part(const float *const *parts, const int64_t *rows, int32_t n_parts) {
    for (int32_t q = 0; q < n_parts; ++q)
        if (rows[q] > 0 && is_pageable(parts[q])) return true;
    return false;
}

// True when kernels on the current device may read pageable host memory in
// place through the host's page tables (Grace-based systems: NVLink-C2C with
// address translation).  Then a copy kernel moves pageable frames at the
// link's rate without host-side staging, and, unlike a cudaMemcpyAsync from
// pageable memory, its launch returns at once.
bool gpu_reads_pageable_host() {
    int dev = 0, pma = 0, pht = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&pht, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return pma == 1 && pht == 1;
}


struct Stager {
    struct Block {
        int64_t row0, rows;
        cudaEvent_t ev = nullptr;
    };
    const float *const *parts = nullptr;
    const int64_t *part_rows = nullptr;
    int32_t n_parts = 0;
    float *X = nullptr;
    int d = 0;
    int device = 0;
    std::vector<Block> blocks;
    std::vector<size_t> chunk_first;  // first block of each chunk (plus blocks.size())
    std::vector<cudaStream_t> streams;
    std::vector<std::thread> threads;
    std::unique_lock<std::mutex> pool_lock;
    std::mutex m;
    std::condition_variable cv;
    std::vector<char> issued;  // per block: its copy is enqueued
    int failed = KM_OK;
    std::string fail_msg;

    // Copies rows [row0, row0 + rows) of the concatenated parts to dst.
    void gather(float *dst, int64_t row0, int64_t rows) const {
        int64_t base = 0;
        for (int32_t q = 0; q < n_parts && rows > 0; ++q) {
            const int64_t r = part_rows[q];
            if (row0 < base + r) {
                const int64_t off = row0 - base, take = std::min(rows, r - off);
                std::memcpy(dst, parts[q] + off * d, sizeof(float) * (size_t)take * d);
                dst += take * d;
                row0 += take;
                rows -= take;
            }
            base += r;
        }
    }

    void worker(int w, int nw, void *buf0, void *buf1) {
        cudaSetDevice(device);
        cudaEvent_t slot_free[2] = {nullptr, nullptr};
        void *buf[2] = {buf0, buf1};
        int use = 0;
        for (size_t b = (size_t)w; b < blocks.size(); b += (size_t)nw, use ^= 1) {
            cudaError_t e = cudaSuccess;
            if (slot_free[use]) e = cudaEventSynchronize(slot_free[use]);  // the slot's last copy is done
            if (e == cudaSuccess) {
                gather(static_cast<float *>(buf[use]), blocks[b].row0, blocks[b].rows);
                e = cudaMemcpyAsync(X + blocks[b].row0 * d, buf[use], sizeof(float) * (size_t)blocks[b].rows * d,
                                    cudaMemcpyHostToDevice, streams[w]);
            }
            if (e == cudaSuccess) e = cudaEventRecord(blocks[b].ev, streams[w]);
            if (e == cudaSuccess) {
                if (!slot_free[use]) e = cudaEventCreateWithFlags(&slot_free[use], cudaEventDisableTiming);
                if (e == cudaSuccess) e = cudaEventRecord(slot_free[use], streams[w]);
            }
            std::lock_guard<std::mutex> lk(m);
            if (e != cudaSuccess && failed == KM_OK) {
                failed = KM_ERR_CUDA;
                fail_msg = std::string("staged host-to-device copy: ") + cudaGetErrorString(e);
            }
            issued[b] = 1;  // also after a failure, so that nobody waits for it forever
            cv.notify_all();
        }
        for (cudaEvent_t ev : slot_free)
            if (ev) {
                cudaEventSynchronize(ev);
                cudaEventDestroy(ev);
            }
    }

    // Splits [0, n) into blocks that never cross a chunk boundary and starts
    // the workers.
    int start(const std::vector<int64_t> &chunk_begin) {
        const int64_t block_rows = std::max<int64_t>(1, (int64_t)(kStageBytes / (sizeof(float) * (size_t)d)));
        for (size_t c = 0; c + 1 < chunk_begin.size(); ++c) {
            chunk_first.push_back(blocks.size());
            for (int64_t a = chunk_begin[c]; a < chunk_begin[c + 1]; a += block_rows)
                blocks.push_back(Block{a, std::min(block_rows, chunk_begin[c + 1] - a)});
        }
        chunk_first.push_back(blocks.size());
        issued.assign(blocks.size(), 0);
        for (Block &b : blocks) KM_CUDA(cudaEventCreateWithFlags(&b.ev, cudaEventDisableTiming));
        const int nw = std::min<int>(stage_workers(), (int)std::max<size_t>(1, blocks.size()));
        StagePool &pool = stage_pool();
        pool_lock = std::unique_lock<std::mutex>(pool.use);
        if (pool.device != device) {
            for (void *p : pool.bufs) cudaFreeHost(p);
            pool.bufs.clear();
            pool.device = device;
        }
        while ((int)pool.bufs.size() < 2 * nw) {
            void *p = nullptr;
            KM_CUDA(cudaHostAlloc(&p, kStageBytes, cudaHostAllocPortable));
            pool.bufs.push_back(p);
        }
        streams.assign(nw, nullptr);
        for (cudaStream_t &st : streams) KM_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        for (int w = 0; w < nw; ++w)
            threads.emplace_back(&Stager::worker, this, w, nw, pool.bufs[2 * w], pool.bufs[2 * w + 1]);
        return KM_OK;
    }

    // Makes st wait for the copies of chunk c (host wait until they are
    // issued, then a device wait on each block's event).
    int wait_chunk(cudaStream_t st, size_t c) {
        {
            std::unique_lock<std::mutex> lk(m);
            cv.wait(lk, [&] {
                for (size_t b = chunk_first[c]; b < chunk_first[c + 1]; ++b)
                    if (!issued[b]) return false;
                return true;
            });
            if (failed != KM_OK) {
                set_error("%s", fail_msg.c_str());
                return failed;
            }
        }
        for (size_t b = chunk_first[c]; b < chunk_first[c + 1]; ++b) KM_CUDA(cudaStreamWaitEvent(st, blocks[b].ev, 0));
        return KM_OK;
    }

    // Joins the workers and waits for every copy (the page-locked ring is
    // free for the next call, the caller's arrays are no longer read).
    int finish() {
        for (std::thread &t : threads)
            if (t.joinable()) t.join();
        threads.clear();
        int st = KM_OK;
        for (cudaStream_t &s : streams) {
            if (s) {
                cudaError_t e = cudaStreamSynchronize(s);
                if (e != cudaSuccess && st == KM_OK) st = cuda_fail(e, "staged copies");
                cudaStreamDestroy(s);
                s = nullptr;
            }
        }
        if (pool_lock.owns_lock()) pool_lock.unlock();
        if (st == KM_OK && failed != KM_OK) {
            set_error("%s", fail_msg.c_str());
            st = failed;
        }
        return st;
    }

    ~Stager() {
        finish();
        for (Block &b : blocks)
            if (b.ev) cudaEventDestroy(b.ev);
    }
};

int lloyd_run(const float *X_in, const HostFrames *hf, int64_t n, int32_t d, int32_t k, float *C, int32_t max_iter,
              double tolerance, int32_t precision, int32_t *labels, double *inertias, int32_t *n_iter,
              int32_t *converged, km_callback cb, void *cb_user, void *workspace, size_t workspace_bytes,
              void *stream, const PairSrc *ps = nullptr) {
    KM_TRY(check_shape(n, d, k));
    if (n < 1 || (!X_in && !ps) || !C || !labels || !n_iter || !converged || max_iter < 0) {
        set_error("Lloyd needs n >= 1, max_iter >= 0 and non-NULL X, C, labels, n_iter, converged");
        return KM_ERR_BAD_SHAPE;
    }
    *n_iter = 0;
    *converged = 0;
    int prec = resolve_precision(precision, d, k, true);
    if (is_tc(prec) && !tc_supported(d, k)) {
        set_error("no tensor-core kernel for d=%d, k=%d on this device", d, k);
        return KM_ERR_UNSUPPORTED;
    }
    const size_t need = lloyd_ws_bytes(n, d, k, prec);
    KM_TRY(check_ws(workspace, workspace_bytes, need));
    if (max_iter == 0 && !hf) return KM_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    float *X = const_cast<float *>(X_in);  // written only by the host-frame copies

    Carver cv(workspace);
    unsigned long long *copy_ctr = cv.take<unsigned long long>(2);
    LoopState *loop_st = cv.take<LoopState>(1);
    double *loop_inertias = cv.take<double>(kLoopBatch);
    void *ws_update = cv.take<char>(update_ws_size(n, d, k));
    float *C_new = cv.take<float>((size_t)k * d);
    double *cost = cv.take<double>(1);
    uint32_t *err = cv.take<uint32_t>(1);
    void *ws_assign = cv.take<char>(assign_ws_bytes(n, d, k, prec));

    // Host frames: one chunked copy on a side stream, an event per chunk.
    struct Streamed {
        cudaStream_t cs = nullptr;
        std::vector<cudaEvent_t> ev;
        std::vector<int64_t> begin;  // first row of each chunk (plus n at the end)
        ~Streamed() {
            for (cudaEvent_t e : ev)
                if (e) cudaEventDestroy(e);
            if (cs) cudaStreamDestroy(cs);
        }
    } sm;
    std::unique_ptr<Stager> stager;  // pageable host frames: staged copies
    if (hf) {
        int64_t total = 0;
        for (int32_t q = 0; q < hf->n_parts; ++q) {
            if (hf->rows[q] < 0 || (hf->rows[q] > 0 && !hf->parts[q])) {
                set_error("host part %d: negative rows or NULL pointer", q);
                return KM_ERR_BAD_SHAPE;
            }
            total += hf->rows[q];
        }
        if (total != n) {
            set_error("host parts hold %lld rows, n = %lld", (long long)total, (long long)n);
            return KM_ERR_BAD_SHAPE;
        }
        const int64_t chunk = stream_chunk_rows(n);
        for (int64_t a = 0; a < n; a += chunk) sm.begin.push_back(a);
        sm.begin.push_back(n);
        if (has_pageable_part(hf->parts, hf->rows, hf->n_parts) && !gpu_reads_pageable_host()) {
            // Workers stage the pageable frames; X must not be in use on s
            // any more (the caller's stream is drained first).
            KM_CUDA(cudaStreamSynchronize(s));
            stager.reset(new Stager());
            stager->parts = hf->parts;
            stager->part_rows = hf->rows;
            stager->n_parts = hf->n_parts;
            stager->X = X;
            stager->d = d;
            KM_CUDA(cudaGetDevice(&stager->device));
            KM_TRY(stager->start(sm.begin));
            if (max_iter == 0) return stager->finish();
        }
    }
    if (hf && !stager) {
        // Where the GPU reads host memory in place, a copy kernel takes every
        // part, page-locked or not: the copy engines' reads of page-locked
        // memory stalled for 10-50 ms in some calls (c3 end to end, 20 calls:
        // mean 25.0 ms, up to 69.6, against 22.4 ms, at most 24.2, by the
        // kernel).  Elsewhere only page-locked parts reach this point, and the
        // copy engines take them.
        const bool in_place = gpu_reads_pageable_host();
        std::vector<char> kernel_copy(hf->n_parts, 0);
        for (int32_t q = 0; q < hf->n_parts; ++q)
            kernel_copy[q] = hf->rows[q] > 0 && (in_place || is_pageable(hf->parts[q]));
        // The copies are the run's critical path: their stream has the
        // device's greatest priority, so their CTAs are placed before the
        // assignment's waiting CTAs whenever an SM has room.
        int least_prio = 0, greatest_prio = 0;
        KM_CUDA(cudaDeviceGetStreamPriorityRange(&least_prio, &greatest_prio));
        KM_CUDA(cudaStreamCreateWithPriority(&sm.cs, cudaStreamNonBlocking, greatest_prio));
        sm.ev.assign(sm.begin.size(), nullptr);  // [0]: the caller's stream reached this call
        for (cudaEvent_t &e : sm.ev) KM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        KM_CUDA(cudaEventRecord(sm.ev[0], s));
        KM_CUDA(cudaStreamWaitEvent(sm.cs, sm.ev[0], 0));
        KM_CUDA(cudaMemsetAsync(copy_ctr, 0, 2 * sizeof(unsigned long long), sm.cs));
        int32_t q = 0;
        int64_t q_off = 0;  // rows of part q already copied
        for (size_t c = 0; c + 1 < sm.begin.size(); ++c) {
            int64_t row = sm.begin[c];
            const int64_t stop = sm.begin[c + 1];
            while (row < stop) {
                while (q < hf->n_parts && q_off == hf->rows[q]) {
                    ++q;
                    q_off = 0;
                }
                const int64_t take = std::min(stop - row, hf->rows[q] - q_off);
                if (kernel_copy[q]) {
                    // read in place by the device (gpu_reads_pageable_host)
                    KM_TRY(launch_host_copy(hf->parts[q] + q_off * d, X + row * d, take * d, copy_ctr, sm.cs));
                } else {
                    KM_CUDA(cudaMemcpyAsync(X + row * d, hf->parts[q] + q_off * d, sizeof(float) * (size_t)take * d,
                                            cudaMemcpyHostToDevice, sm.cs));
                }
                row += take;
                q_off += take;
            }
            KM_CUDA(cudaEventRecord(sm.ev[c + 1], sm.cs));
        }
        if (max_iter == 0) {
            KM_CUDA(cudaStreamWaitEvent(s, sm.ev.back(), 0));
            KM_CUDA(cudaStreamSynchronize(s));
            return KM_OK;
        }
    }

    // Tensor-core iterations run the exact re-check on a side stream beside
    // the centroid update, which sums by the tensor-core labels; the frames
    // whose exact label differs then move between clusters before the new
    // centers are formed.
    FlipList fl;
    struct Side {
        cudaStream_t st = nullptr;
        cudaEvent_t fork[kTcMaxChunks] = {}, join = nullptr;
        ~Side() {
            for (cudaEvent_t e : fork)
                if (e) cudaEventDestroy(e);
            if (join) cudaEventDestroy(join);
            if (st) cudaStreamDestroy(st);
        }
    } side;
    if (is_tc(prec)) {
        fl.rows = cv.take<int32_t>(3 * (size_t)n);
        fl.count = cv.take<int32_t>(1);
        fl.cap = n;
        KM_CUDA(cudaStreamCreateWithFlags(&side.st, cudaStreamNonBlocking));
        for (cudaEvent_t &e : side.fork) KM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        KM_CUDA(cudaEventCreateWithFlags(&side.join, cudaEventDisableTiming));
    }

    TcBuffers b;
    if (is_tc(prec)) {
        // The shift and scale stay fixed for the whole run so that the 16-bit
        // frame copy is made once.
        carve_assign(ws_assign, n, d, k, b);
        tc_set_operand(b, d, prec);
        KM_TRY(tc_prepare_shift_from_centers(C, d, k, b, s));
        if (!hf) KM_TRY(tc_prepare_frames(X, n, d, b, s, ps));
    }
    KM_CUDA(cudaMemsetAsync(err, 0, sizeof(uint32_t), s));

    // One iteration: assign, update, C <- C_new.  The first iteration runs
    // eagerly (it also performs every lazy one-time set-up); the following
    // ones replay a CUDA graph captured from the same sequence.  With host
    // frames the first iteration assigns each chunk as soon as its copy has
    // landed (and makes its 16-bit copy first), overlapping the transfer.
    ProfEvents prof;
    KM_TRY(prof.open());
    struct Closer {
        ProfEvents &p;
        ~Closer() { p.close(); }
    } closer{prof};
    auto enqueue_update = [&](cudaStream_t st) -> int {
        prof.begin(kProfUpdate, st);
        KM_TRY(launch_update(X, n, d, labels, k, C, C_new, nullptr, cost, err, ws_update, st, ps));
        prof.end(kProfUpdate, st);
        KM_CUDA(cudaMemcpyAsync(C, C_new, sizeof(float) * k * d, cudaMemcpyDeviceToDevice, st));
        return KM_OK;
    };
    auto enqueue = [&](cudaStream_t st) -> int {
        if (is_tc(prec)) {
            KM_TRY(tc_prepare_centers(C, d, k, b, st));
            KM_CUDA(cudaMemsetAsync(fl.count, 0, sizeof(int32_t), st));
            // the tensor-core pass counts the members as it writes the labels
            int32_t *counts = update_counts_from_labels(d, k, ps) ? update_counts(ws_update, n, d, k) : nullptr;
            if (counts) KM_CUDA(cudaMemsetAsync(counts, 0, sizeof(int32_t) * k, st));
            KM_TRY(tc_assign_deferred(X, n, d, C, k, labels, b, st, side.st, side.fork, kTcMaxChunks, fl, &prof, ps,
                                      counts));
            prof.begin(kProfUpdate, st);
            // one segment-sum CTA per SM: room for the re-check beside it
            KM_TRY(launch_update_accumulate(X, n, d, labels, k, C, err, ws_update, st, 1, ps, counts != nullptr));
            KM_CUDA(cudaEventRecord(side.join, side.st));
            KM_CUDA(cudaStreamWaitEvent(st, side.join, 0));
            KM_TRY(launch_apply_flips(X, n, d, k, C, fl, labels, ws_update, st, ps));
            KM_TRY(launch_update_finish(n, d, k, C, C_new, nullptr, cost, ws_update, st));
            prof.end(kProfUpdate, st);
            KM_CUDA(cudaMemcpyAsync(C, C_new, sizeof(float) * k * d, cudaMemcpyDeviceToDevice, st));
            return KM_OK;
        } else {
            prof.begin(kProfFp32, st);
            KM_TRY(launch_assign_fp32(X, nullptr, nullptr, n, d, C, k, labels, nullptr, nullptr, st, ps));
            prof.end(kProfFp32, st);
        }
        return enqueue_update(st);
    };
    auto enqueue_streamed = [&](cudaStream_t st) -> int {
        if (is_tc(prec)) {
            KM_TRY(tc_prepare_centers(C, d, k, b, st));
            KM_CUDA(cudaMemsetAsync(b.err, 0, sizeof(uint32_t), st));
        }
        // Each chunk's members join the update's sums as soon as the chunk
        // is assigned, so only the division remains after the last copy.
        prof.begin(kProfUpdate, st);
        KM_TRY(launch_update_parts_begin(n, d, k, ws_update, st));
        for (size_t c = 0; c + 1 < sm.begin.size(); ++c) {
            const int64_t a = sm.begin[c], rows = sm.begin[c + 1] - a;
            if (stager)
                KM_TRY(stager->wait_chunk(st, c));
            else
                KM_CUDA(cudaStreamWaitEvent(st, sm.ev[c + 1], 0));
            if (is_tc(prec)) {
                TcBuffers v = tc_rows_from(b, a);
                v.keep_err = 1;
                KM_TRY(tc_prepare_frames(X + a * d, rows, d, v, st));
                KM_TRY(tc_assign(X + a * d, rows, d, C, k, labels + a, v, st, &prof));
            } else {
                prof.begin(kProfFp32, st);
                KM_TRY(launch_assign_fp32(X + a * d, nullptr, nullptr, rows, d, C, k, labels + a, nullptr, nullptr,
                                          st));
                prof.end(kProfFp32, st);
            }
            KM_TRY(launch_update_part(X + a * d, n, d, labels + a, rows, k, C, err, ws_update, st));
        }
        KM_TRY(launch_update_parts_finish(n, d, k, C, C_new, cost, ws_update, st));
        prof.end(kProfUpdate, st);
        KM_CUDA(cudaMemcpyAsync(C, C_new, sizeof(float) * k * d, cudaMemcpyDeviceToDevice, st));
        return KM_OK;
    };

    // The iterations it0, it0+1, ... as device-side WHILE loops.  handled = 0
    // when the graph could not be built (then the host loop runs them).
    auto device_loop = [&](int32_t it0, double prev0, int &handled) -> int {
        handled = 0;
        cudaStream_t cs = nullptr;
        cudaGraph_t g = nullptr;
        cudaGraphExec_t gx = nullptr;
        auto cleanup = [&]() {
            if (gx) cudaGraphExecDestroy(gx);
            if (g) cudaGraphDestroy(g);
            if (cs) cudaStreamDestroy(cs);
        };
        bool ok = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess;
        if (ok) ok = cudaGraphCreate(&g, 0) == cudaSuccess;
        cudaGraphConditionalHandle h = 0;
        if (ok) ok = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
        cudaGraphNodeParams np = {};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        if (ok) ok = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np) == cudaSuccess;
        if (ok) {
            cudaGraph_t body = np.conditional.phGraph_out[0];
            ok = cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
                 cudaSuccess;
            if (ok) {
                const int st = enqueue(cs);
                lloyd_loop_step_kernel<<<1, 1, 0, cs>>>(loop_st, cost, err, is_tc(prec) ? b.err : nullptr,
                                                        loop_inertias, h);
                cudaGraph_t out = nullptr;
                const cudaError_t e2 = cudaStreamEndCapture(cs, &out);
                ok = st == KM_OK && e2 == cudaSuccess;
            }
        }
        if (ok) ok = instantiate_with_priorities(&gx, g) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();  // not fatal: the host loop takes over
            cleanup();
            return KM_OK;
        }
        handled = 1;
        int status = KM_OK;
        int32_t it = it0;
        double prev = prev0;
        while (it < max_iter) {
            LoopState hs{prev, tolerance, 0, std::min(kLoopBatch, max_iter - it), 0, 0u};
            double hin[kLoopBatch];
            cudaError_t e = cudaMemcpyAsync(loop_st, &hs, sizeof(hs), cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = cudaGraphLaunch(gx, s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, loop_st, sizeof(hs), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(hin, loop_inertias, sizeof(double) * kLoopBatch, cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) {
                status = cuda_fail(e, "Lloyd iterations");
                break;
            }
            for (int32_t j = 0; j < hs.it; ++j)
                if (inertias) inertias[it + j] = hin[j];
            it += hs.it;
            *n_iter = it;
            if (hs.it > 0) prev = hin[hs.it - 1];
            status = check_device_errors(hs.err);
            if (status != KM_OK) break;
            if (hs.converged) {
                *converged = 1;
                break;
            }
            if (hs.it == 0) break;
        }
        cleanup();
        return status;
    };

    cudaGraphExec_t exec = nullptr;
    int status = KM_OK;
    double prev = 0.0;
    for (int32_t it = 0; it < max_iter; ++it) {
        if (it == 1 && !cb && !prof.active) {
            int handled = 0;
            status = device_loop(it, prev, handled);
            if (handled || status != KM_OK) break;
        }
        if (it == 0) {
            status = hf ? enqueue_streamed(s) : enqueue(s);
        } else {
            if (!exec) {
                cudaStream_t cs;
                KM_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
                cudaGraph_t graph = nullptr;
                cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
                if (e == cudaSuccess) {
                    status = enqueue(cs);
                    cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
                    if (status == KM_OK && e2 != cudaSuccess) status = cuda_fail(e2, "cudaStreamEndCapture");
                    if (status == KM_OK) {
                        e2 = instantiate_with_priorities(&exec, graph);
                        if (e2 != cudaSuccess) status = cuda_fail(e2, "cudaGraphInstantiate");
                    }
                    if (graph) cudaGraphDestroy(graph);
                } else {
                    status = cuda_fail(e, "cudaStreamBeginCapture");
                }
                cudaStreamDestroy(cs);
                if (status != KM_OK) break;
            }
            cudaError_t e = cudaGraphLaunch(exec, s);
            if (e != cudaSuccess) {
                status = cuda_fail(e, "cudaGraphLaunch");
                break;
            }
        }
        if (status != KM_OK) break;
        double h_cost = 0.0;
        uint32_t h_err = 0, tc_err = 0;
        cudaError_t e = cudaMemcpyAsync(&h_cost, cost, sizeof(double), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&h_err, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && is_tc(prec))
            e = cudaMemcpyAsync(&tc_err, b.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            status = cuda_fail(e, "Lloyd iteration");
            break;
        }
        h_err |= tc_err;
        prof.collect();
        status = check_device_errors(h_err);
        if (status != KM_OK) break;
        if (inertias) inertias[it] = h_cost;
        *n_iter = it + 1;
        const double rel = h_cost != 0.0 ? fabs(h_cost - prev) / h_cost : 0.0;
        prev = h_cost;
        if (cb) cb(cb_user);
        if (rel <= tolerance) {
            *converged = 1;
            break;
        }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (stager) {
        const int st2 = stager->finish();
        if (status == KM_OK) status = st2;
    } else if (hf && status != KM_OK) {
        // The copies may still be running into X: wait for them before
        // returning the caller's buffer.
        cudaStreamSynchronize(sm.cs);
    }
    return status;
}

}  // namespace

extern "C" {

int km_lloyd(const float *X, int64_t n, int32_t d, int32_t k, float *C, int32_t max_iter, double tolerance,
             int32_t precision, int32_t *labels, double *inertias, int32_t *n_iter, int32_t *converged,
             km_callback cb, void *cb_user, void *workspace, size_t workspace_bytes, void *stream) {
    return lloyd_run(X, nullptr, n, d, k, C, max_iter, tolerance, precision, labels, inertias, n_iter, converged, cb,
                     cb_user, workspace, workspace_bytes, stream);
}

// ---- frames given as atom coordinates (the featurization fused in) ---------

namespace {
int check_pair_args(const float *xyz, int64_t n, int32_t n_atoms, const int32_t *pairs, int32_t d,
                    cudaStream_t s) {
    if (n_atoms < 1 || (n > 0 && !xyz) || !pairs) {
        set_error("coordinates need n_atoms >= 1 and non-NULL xyz and pairs");
        return KM_ERR_BAD_SHAPE;
    }
    return check_pairs(pairs, d, n_atoms, s);
}
}  // namespace

size_t km_assign_pairs_workspace_size(int64_t n, int32_t d, int32_t k, int32_t precision) {
    return km_assign_workspace_size(n, d, k, precision);
}

int km_assign_pairs(const float *xyz, int64_t n, int32_t n_atoms, const int32_t *pairs, int32_t d, const float *C,
                    int32_t k, int32_t precision, int32_t *labels, void *workspace, size_t workspace_bytes,
                    km_assign_stats *stats, void *stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    KM_TRY(check_shape(n, d, k));
    KM_TRY(check_pair_args(xyz, n, n_atoms, pairs, d, s));
    PairSrc ps;
    ps.xyz = xyz;
    ps.pairs = pairs;
    ps.n_atoms = n_atoms;
    return assign_impl(nullptr, n, d, C, k, precision, labels, workspace, workspace_bytes, stats, s, &ps);
}

size_t km_lloyd_pairs_workspace_size(int64_t n, int32_t d, int32_t k, int32_t precision) {
    return km_lloyd_workspace_size(n, d, k, precision);
}

int km_lloyd_pairs(const float *xyz, int64_t n, int32_t n_atoms, const int32_t *pairs, int32_t d, int32_t k,
                   float *C, int32_t max_iter, double tolerance, int32_t precision, int32_t *labels,
                   double *inertias, int32_t *n_iter, int32_t *converged, km_callback cb, void *cb_user,
                   void *workspace, size_t workspace_bytes, void *stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    KM_TRY(check_shape(n, d, k));
    KM_TRY(check_pair_args(xyz, n, n_atoms, pairs, d, s));
    if (resolve_precision(precision, d, k, true) == KM_PREC_FP8) {
        set_error("FP8 operands are not built for coordinate frames");
        return KM_ERR_UNSUPPORTED;
    }
    PairSrc ps;
    ps.xyz = xyz;
    ps.pairs = pairs;
    ps.n_atoms = n_atoms;
    return lloyd_run(nullptr, nullptr, n, d, k, C, max_iter, tolerance, precision, labels, inertias, n_iter, converged,
                     cb, cb_user, workspace, workspace_bytes, stream, &ps);
}

size_t km_kmpp_pairs_workspace_size(int64_t n, int32_t d, int32_t k) { return km_kmpp_workspace_size(n, d, k); }

int km_kmpp_pairs(const float *xyz, int64_t n, int32_t n_atoms, const int32_t *pairs, int32_t d, int32_t k,
                  uint32_t seed, float *C0, int64_t *idx, km_callback cb, void *cb_user, void *workspace,
                  size_t workspace_bytes, void *stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    KM_TRY(check_shape(n, d, k));
    if (n < 1 || !C0) {
        set_error("kmeans++ needs n >= 1 and non-NULL C0");
        return KM_ERR_BAD_SHAPE;
    }
    KM_TRY(check_pair_args(xyz, n, n_atoms, pairs, d, s));
    KM_TRY(check_ws(workspace, workspace_bytes, kmpp_ws_size(n, d, k)));
    PairSrc ps;
    ps.xyz = xyz;
    ps.pairs = pairs;
    ps.n_atoms = n_atoms;
    return run_kmpp(nullptr, n, d, k, seed, C0, idx, cb, cb_user, workspace, s, nullptr, &ps);
}

int km_lloyd_host(const float *const *X_parts, const int64_t *part_rows, int32_t n_parts, float *X, int64_t n,
                  int32_t d, int32_t k, float *C, int32_t max_iter, double tolerance, int32_t precision,
                  int32_t *labels, double *inertias, int32_t *n_iter, int32_t *converged, km_callback cb,
                  void *cb_user, void *workspace, size_t workspace_bytes, void *stream) {
    if (n_parts < 0 || (n_parts > 0 && (!X_parts || !part_rows))) {
        set_error("km_lloyd_host needs n_parts >= 0 with X_parts and part_rows");
        return KM_ERR_BAD_SHAPE;
    }
    HostFrames hf{X_parts, part_rows, n_parts};
    return lloyd_run(X, &hf, n, d, k, C, max_iter, tolerance, precision, labels, inertias, n_iter, converged, cb,
                     cb_user, workspace, workspace_bytes, stream);
}

// ---- resident center sets --------------------------------------------------

int km_centers_create(const float *C, int32_t k, int32_t d, int32_t precision, void *stream, km_centers **out) {
    if (!out) {
        set_error("out must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    *out = nullptr;
    KM_TRY(check_shape(0, d, k));
    if (!C) {
        set_error("C must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    const int prec = resolve_precision(precision, d, k, true);
    if (prec != KM_PREC_FP32 && !is_tc(prec)) {
        set_error("unknown precision %d", precision);
        return KM_ERR_BAD_SHAPE;
    }
    if (is_tc(prec) && !tc_supported(d, k)) {
        set_error("no tensor-core kernel for d=%d, k=%d on this device", d, k);
        return KM_ERR_UNSUPPORTED;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    km_centers *h = new km_centers();
    h->k = k;
    h->d = d;
    h->prec = prec;
    cudaGetDevice(&h->device);
    const size_t c_bytes = ((size_t)k * d * sizeof(float) + 255) / 256 * 256;
    h->bytes = c_bytes + (is_tc(prec) ? tc_centers_ws_size(d, k) : 0);
    cudaError_t e = cudaMalloc(&h->mem, h->bytes);
    if (e != cudaSuccess) {
        delete h;
        return cuda_fail(e, "cudaMalloc (resident centers)");
    }
    h->C = static_cast<float *>(h->mem);
    int st = KM_OK;
    e = cudaMemcpyAsync(h->C, C, (size_t)k * d * sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) st = cuda_fail(e, "cudaMemcpyAsync (resident centers)");
    if (st == KM_OK && is_tc(prec)) {
        tc_carve_centers(static_cast<char *>(h->mem) + c_bytes, d, k, h->tc);
        tc_set_operand(h->tc, d, prec);
        st = tc_prepare_shift_from_centers(h->C, d, k, h->tc, s);
        if (st == KM_OK) st = tc_prepare_centers(h->C, d, k, h->tc, s);
    }
    if (st == KM_OK) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = cuda_fail(e, "cudaStreamSynchronize (resident centers)");
    }
    if (st != KM_OK) {
        cudaFree(h->mem);
        delete h;
        return st;
    }
    *out = h;
    return KM_OK;
}

int km_centers_destroy(km_centers *h) {
    if (!h) return KM_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    if (prev != h->device) cudaSetDevice(h->device);
    cudaError_t e = cudaFree(h->mem);
    if (prev != h->device) cudaSetDevice(prev);
    delete h;
    if (e != cudaSuccess) return cuda_fail(e, "cudaFree (resident centers)");
    return KM_OK;
}

int km_centers_info(const km_centers *h, int32_t *k, int32_t *d, int32_t *precision, int64_t *device_bytes) {
    if (!h) {
        set_error("centers must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    if (k) *k = h->k;
    if (d) *d = h->d;
    if (precision) *precision = h->prec;
    if (device_bytes) *device_bytes = (int64_t)h->bytes;
    return KM_OK;
}

size_t km_assign_centers_workspace_size(int64_t n, const km_centers *h) {
    if (!h || check_shape(n, h->d, h->k) != KM_OK) return 0;
    return resident_ws_bytes(n, h->d, h->k, h->prec);
}

int km_assign_centers(const float *X, int64_t n, int32_t d, const km_centers *h, int32_t *labels, void *workspace,
                      size_t workspace_bytes, km_assign_stats *stats, void *stream) {
    if (!h) {
        set_error("centers must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    KM_TRY(check_shape(n, d, h->k));
    if (d != h->d) {
        set_error("frames have d=%d, the center set d=%d", d, h->d);
        return KM_ERR_BAD_SHAPE;
    }
    if (n > 0 && (!X || !labels)) {
        set_error("X and labels must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    KM_TRY(check_ws(workspace, workspace_bytes, resident_ws_bytes(n, d, h->k, h->prec)));
    TcBuffers b;
    if (is_tc(h->prec) && n > 0) {
        b = h->tc;  // prepared center half; the carves below fill the frame and list fields
        char *p = static_cast<char *>(workspace);
        tc_carve_frames(p, n, d, b);
        p += (tc_frames_ws_size(n, d) + 255) / 256 * 256;
        tc_carve_assign(p, n, d, h->k, b);
        tc_set_operand(b, d, h->prec);
    }
    return assign_core(X, n, d, h->C, h->k, h->prec, labels, b, true, stats, static_cast<cudaStream_t>(stream));
}

// ---- precision autotuning ----------------------------------------------------

size_t km_tune_workspace_size(int64_t n, int32_t d, int32_t k) {
    if (check_shape(n, d, k) != KM_OK) return 0;
    Carver c(nullptr);
    c.take<int32_t>(n > 0 ? n : 1);
    c.take<char>(assign_ws_bytes(n, d, k, KM_PREC_FP16));
    return c.bytes();
}

int km_tune(const float *X, int64_t n, int32_t d, const float *C, int32_t k, void *workspace,
            size_t workspace_bytes, int32_t *chosen, double *ms_fp32, double *ms_fp16, void *stream) {
    KM_TRY(check_shape(n, d, k));
    if (n < 1 || !X || !C) {
        set_error("km_tune needs n >= 1 and non-NULL X, C");
        return KM_ERR_BAD_SHAPE;
    }
    KM_TRY(check_ws(workspace, workspace_bytes, km_tune_workspace_size(n, d, k)));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) == cudaSuccess && cap != cudaStreamCaptureStatusNone) {
        set_error("km_tune synchronises and cannot run while the stream is captured");
        return KM_ERR_BAD_SHAPE;
    }
    Carver cv(workspace);
    int32_t *labels = cv.take<int32_t>(n);
    void *ws = cv.take<char>(assign_ws_bytes(n, d, k, KM_PREC_FP16));
    const size_t ws_bytes = assign_ws_bytes(n, d, k, KM_PREC_FP16);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    KM_CUDA(cudaEventCreate(&e0));
    cudaError_t ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) {
        cudaEventDestroy(e0);
        return cuda_fail(ce, "cudaEventCreate");
    }
    // Median-free timing: one warm-up call, then the mean of three.
    auto time_prec = [&](int prec, double *ms) -> int {
        KM_TRY(assign_impl(X, n, d, C, k, prec, labels, ws, ws_bytes, nullptr, s));
        KM_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < 3; ++r) KM_TRY(assign_impl(X, n, d, C, k, prec, labels, ws, ws_bytes, nullptr, s));
        KM_CUDA(cudaEventRecord(e1, s));
        KM_CUDA(cudaEventSynchronize(e1));
        float t = 0.0f;
        KM_CUDA(cudaEventElapsedTime(&t, e0, e1));
        *ms = t / 3.0;
        return KM_OK;
    };
    double t32 = 0.0, t16 = -1.0;
    int st = time_prec(KM_PREC_FP32, &t32);
    const bool tc_ok = tc_supported(d, k);
    if (st == KM_OK && tc_ok) st = time_prec(KM_PREC_FP16, &t16);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != KM_OK) return st;
    const int best = (tc_ok && t16 < t32) ? KM_PREC_FP16 : KM_PREC_FP32;
    {
        std::lock_guard<std::mutex> lk(g_tune.m);
        g_tune.choice[std::make_pair((int)d, (int)k)] = best;
    }
    if (chosen) *chosen = best;
    if (ms_fp32) *ms_fp32 = t32;
    if (ms_fp16) *ms_fp16 = t16;
    return KM_OK;
}

namespace {
// Clears the thread's forced tile shape when a tuning call returns.
struct ForcedPlanGuard {
    ~ForcedPlanGuard() { tc_force_plan(nullptr); }
};
thread_local TilePlan t_debug_plan;
}  // namespace

int km_tune_tiles(const float *X, int64_t n, int32_t d, const float *C, int32_t k, int32_t precision,
                  void *workspace, size_t workspace_bytes, km_tile_plan *best, km_tile_plan *tried,
                  int32_t max_tried, int32_t *n_tried, void *stream) {
    KM_TRY(check_shape(n, d, k));
    if (n < 1 || !X || !C || !best) {
        set_error("km_tune_tiles needs n >= 1 and non-NULL X, C, best");
        return KM_ERR_BAD_SHAPE;
    }
    if (precision != KM_PREC_FP16 && precision != KM_PREC_BF16) {
        set_error("km_tune_tiles tunes the tensor-core precisions (KM_PREC_FP16, KM_PREC_BF16)");
        return KM_ERR_BAD_SHAPE;
    }
    if (!tc_supported(d, k)) {
        set_error("no tensor-core kernel for d=%d, k=%d on this device", d, k);
        return KM_ERR_UNSUPPORTED;
    }
    KM_TRY(check_ws(workspace, workspace_bytes, km_tune_workspace_size(n, d, k)));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) == cudaSuccess && cap != cudaStreamCaptureStatusNone) {
        set_error("km_tune_tiles synchronises and cannot run while the stream is captured");
        return KM_ERR_BAD_SHAPE;
    }
    std::vector<TilePlan> cands;
    tc_enumerate_plans(d, k, cands);
    if (cands.empty()) {
        set_error("no tile shape fits d=%d, k=%d", d, k);
        return KM_ERR_UNSUPPORTED;
    }
    Carver cv(workspace);
    int32_t *labels = cv.take<int32_t>(n);
    const size_t ws_bytes = assign_ws_bytes(n, d, k, KM_PREC_FP16);
    void *ws = cv.take<char>(ws_bytes);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    KM_CUDA(cudaEventCreate(&e0));
    cudaError_t ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) {
        cudaEventDestroy(e0);
        return cuda_fail(ce, "cudaEventCreate");
    }
    ForcedPlanGuard guard;
    int st = KM_OK;
    int ibest = -1;
    double tbest = 0.0;
    if (n_tried) *n_tried = 0;
    for (size_t c = 0; c < cands.size() && st == KM_OK; ++c) {
        tc_force_plan(&cands[c]);
        // one warm-up call, then the mean of three
        st = assign_impl(X, n, d, C, k, precision, labels, ws, ws_bytes, nullptr, s);
        if (st == KM_OK) st = cudaEventRecord(e0, s) == cudaSuccess ? KM_OK : KM_ERR_CUDA;
        for (int r = 0; r < 3 && st == KM_OK; ++r)
            st = assign_impl(X, n, d, C, k, precision, labels, ws, ws_bytes, nullptr, s);
        float t = 0.0f;
        if (st == KM_OK) {
            cudaError_t e = cudaEventRecord(e1, s);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
            if (e != cudaSuccess) st = cuda_fail(e, "timing a tile shape");
        }
        if (st != KM_OK) break;
        const double ms = t / 3.0;
        if (tried && n_tried && *n_tried < max_tried) {
            tried[*n_tried] = km_tile_plan{cands[c].bn, cands[c].pair, cands[c].stages, cands[c].list_len, ms};
            *n_tried += 1;
        }
        if (ibest < 0 || ms < tbest) {
            ibest = (int)c;
            tbest = ms;
        }
    }
    tc_force_plan(nullptr);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != KM_OK) return st;
    const TilePlan &b = cands[ibest];
    tc_store_plan(d, k, b);
    *best = km_tile_plan{b.bn, b.pair, b.stages, b.list_len, tbest};
    return KM_OK;
}

int km_tile_plan_get(int32_t d, int32_t k, km_tile_plan *plan, int32_t *tuned) {
    KM_TRY(check_shape(1, d, k));
    if (!plan) {
        set_error("plan must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    TilePlan tp;
    bool tu = false;
    if (!tc_current_plan(d, k, &tp, &tu)) {
        set_error("no tile shape fits d=%d, k=%d", d, k);
        return KM_ERR_UNSUPPORTED;
    }
    *plan = km_tile_plan{tp.bn, tp.pair, tp.stages, tp.list_len, 0.0};
    if (tuned) *tuned = tu ? 1 : 0;
    return KM_OK;
}

int km_debug_force_tile_plan(const km_tile_plan *plan) {
    if (!plan) {
        tc_force_plan(nullptr);
        return KM_OK;
    }
    t_debug_plan = TilePlan{plan->bn, plan->pair, plan->stages, plan->list_len};
    tc_force_plan(&t_debug_plan);
    return KM_OK;
}

int km_tune_clear(void) {
    std::lock_guard<std::mutex> lk(g_tune.m);
    g_tune.choice.clear();
    tc_clear_plans();
    return KM_OK;
}

}  // extern "C"

namespace km {

bool gpu_reads_host_in_place() { return gpu_reads_pageable_host(); }

int launch_host_copy(const float *src, float *dst, int64_t count, unsigned long long *ctr, cudaStream_t s) {
    if (count <= 0) return KM_OK;
    const int64_t g = std::min<int64_t>((count + kCopyBlock - 1) / kCopyBlock, (int64_t)num_sms());
    host_copy_kernel<<<(unsigned)(g < 1 ? 1 : g), kCopyThreads, 0, s>>>(src, dst, count, ctr);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

}  // namespace km

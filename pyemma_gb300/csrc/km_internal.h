// km_internal.h -- host launchers shared between the translation units of
// libkmgpu.  Not part of the public ABI (include/kmgpu.h is).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstddef>
#include <vector>

#include "../../include/kmgpu.h"

namespace km {

// Frames given as atom coordinates: feature f of frame i is the distance
// between atoms pairs[2f] and pairs[2f+1] of xyz[i] (device arrays).  The
// launchers below take a nullable PairSrc; when it is set, X is ignored and
// every float32 feature is computed from the coordinates where it is read.
struct PairSrc {
    const float *xyz = nullptr;   // (n, n_atoms, 3)
    const int32_t *pairs = nullptr;  // (d, 2)
    int n_atoms = 0;
};

// featurize.cu: KM_ERR_BAD_SHAPE unless every atom index of the pairs (device,
// npairs x 2) lies in [0, n_atoms); synchronises s.
int check_pairs(const int32_t *pairs, int32_t npairs, int32_t n_atoms, cudaStream_t s);

// ---- profiling (capi.cu) ------------------------------------------------------
// Event pairs recorded around the main kernels of one pass when profiling is
// on (km_profile_enable).  Inside a captured graph the records become event
// nodes, so every replay re-times the same launches.
enum ProfKind { kProfTc = 0, kProfFp32 = 1, kProfRecheck = 2, kProfUpdate = 3, kProfFull = 4, kProfKinds = 5 };

struct ProfEvents {
    cudaEvent_t ev[kProfKinds][2] = {};
    bool used[kProfKinds] = {};
    bool active = false;
    int open();                 // creates the events when profiling is on
    void close();
    void begin(int kind, cudaStream_t s);
    void end(int kind, cudaStream_t s);
    void collect();             // after a synchronisation: adds elapsed times to the totals
};

// ---- assign_fp32.cu ------------------------------------------------------
// Exact float32 argmin over all k centers.  With frame_idx the kernel visits
// frames frame_idx[0..n) and writes labels[frame_idx[i]]; n_dev (nullable)
// replaces n by a device-resident count capped at n.  flipped (nullable)
// counts frames whose new label differs from the one already in labels.
int launch_assign_fp32(const float *X, const int32_t *frame_idx, const int32_t *n_dev, int64_t n,
                       int d, const float *C, int k, int32_t *labels, float *dist,
                       unsigned long long *flipped, cudaStream_t s, const PairSrc *ps = nullptr);

// Labels that an exact re-check changes, listed instead of written: entry i
// is (frame, label before, exact label) at rows[3i..3i+2]; *count (device)
// counts them (at most cap).  A Lloyd iteration lets the centroid update run
// on the tensor-core labels while the re-check runs beside it, then moves the
// listed frames between clusters (launch_apply_flips).
struct FlipList {
    int32_t *rows = nullptr;
    int32_t *count = nullptr;
    int64_t cap = 0;
};

// Exact re-evaluation of the frames frames[0..*n_dev) against all centers,
// split over (frame tile, center block) CTAs; keys[e] must hold ~0 on entry.
// With fl the changed labels go to the list and labels stays as it is.
int launch_full_recheck(const float *X, const int32_t *frames, const int32_t *n_dev, int64_t n_max, int d,
                        const float *C, int k, unsigned long long *keys, int32_t *labels,
                        unsigned long long *flipped, cudaStream_t s, const FlipList *fl = nullptr,
                        const PairSrc *ps = nullptr);

// Re-evaluation of the candidates the tensor-core kernel could not
// separate.  Entry e stands for frame rc_frames[e]; its candidates are the
// pairs rc_pairs[e] >> 8 .. + (rc_pairs[e] & 255) (centers pair_center[q],
// tensor-core lower bounds pair_lo[q]), rc_best[e] the one with the best
// tensor-core value.  A warp per entry evaluates them in float32 with
// coalesced loads; the bracket of that sum settles most entries, and the
// rest (amb_entries / amb_mask, counters[3]) get the exact float32 distance
// of their remaining candidates in feature order, the minimum collected in
// keys[e] (initialised to ~0).  counters[0] = entries (device).  With fl the
// changed labels go to the list and labels stays as it is.
int launch_recheck_pairs(const float *X, int d, const float *C, const int32_t *rc_frames, const int32_t *rc_best,
                         const int64_t *rc_pairs, const int32_t *pair_center, const float *pair_lo,
                         unsigned long long *keys, int32_t *amb_entries, int32_t *amb_mask, int32_t *counters,
                         int64_t max_entries, int32_t *labels, unsigned long long *flipped, cudaStream_t s,
                         const FlipList *fl = nullptr, int blocks_per_sm = 8, const PairSrc *ps = nullptr);

// ---- update.cu -------------------------------------------------------------
size_t update_ws_size(int64_t n, int d, int k);
// Enqueues one centroid update (no host synchronisation).  err (device,
// uint32) receives kDevBadLabel when a label is outside [0, k).
int launch_update(const float *X, int64_t n, int d, const int32_t *labels, int k,
                  const float *C_old, float *C_new, int64_t *counts_out, double *cost,
                  uint32_t *err, void *ws, cudaStream_t s, const PairSrc *ps = nullptr);
// launch_update in two halves: the sums over the members (counting sort and
// segment sums) and the new centers and inertia from those sums.
// seg_per_sm > 0 caps the segment-sum CTAs per SM (room for a kernel beside it).
// counted: the member counts of `labels` are already in the workspace (added
// by the tensor-core pass into update_counts(), cleared before it); only
// valid where update_counts_from_labels() holds.
int launch_update_accumulate(const float *X, int64_t n, int d, const int32_t *labels, int k, const float *C_old,
                             uint32_t *err, void *ws, cudaStream_t s, int seg_per_sm = 0,
                             const PairSrc *ps = nullptr, bool counted = false);
// The member-count array of an update workspace, and whether the update of
// (d, k) counts its members from the labels in a pass of its own (the
// counting-sort path; the one-pass small-shape path counts as it sums).
int32_t *update_counts(void *ws, int64_t n, int d, int k);
bool update_counts_from_labels(int d, int k, const PairSrc *ps);
int launch_update_finish(int64_t n, int d, int k, const float *C_old, float *C_new, int64_t *counts_out,
                         double *cost, void *ws, cudaStream_t s);
// The update of frames that arrive in parts: begin clears the totals, each
// part adds its rows (X, labels already offset to the part; n is the full
// count the workspace was sized for), finish forms the new centers and the
// inertia.  The result equals launch_update over all rows up to the order
// of the float64 sums.
int launch_update_parts_begin(int64_t n, int d, int k, void *ws, cudaStream_t s);
int launch_update_part(const float *X, int64_t n, int d, const int32_t *labels, int64_t rows, int k,
                       const float *C_old, uint32_t *err, void *ws, cudaStream_t s);
int launch_update_parts_finish(int64_t n, int d, int k, const float *C_old, float *C_new, double *cost, void *ws,
                               cudaStream_t s);
// Between the halves: moves the frames of a flip list from the cluster of
// their first label to that of their exact label (sums, squared sums, counts,
// with the accumulation's float32 deviations) and writes the exact labels.
int launch_apply_flips(const float *X, int64_t n, int d, int k, const float *C_old, const FlipList &fl,
                       int32_t *labels, void *ws, cudaStream_t s, const PairSrc *ps = nullptr);

// ---- kmpp.cu -----------------------------------------------------------------
size_t kmpp_ws_size(int64_t n, int d, int k);
// D^2 of kmeans++ under the minRMSD metric: the centered frames Xc with
// their traces G; idx (device, k) receives the chosen frames and names the
// newest center of each round.
struct KmppMetric {
    const float *Xc;
    const double *G;
    const int64_t *idx;
};
int run_kmpp(const float *X, int64_t n, int d, int k, uint32_t seed, float *C0, int64_t *idx,
             void (*cb)(void *), void *cb_user, void *ws, cudaStream_t s, const KmppMetric *metric = nullptr,
             const PairSrc *ps = nullptr);


// ---- assign_tc.cu ------------------------------------------------------------
// Tensor-core (tcgen05, FP16 operands) assignment with exact FP32 recheck.
bool tc_supported(int d, int k);   // a plan exists and the device is sm_10x
bool tc_plan_exists(int d, int k); // shape check only (no device query)

// Tile shape of the tensor-core kernel: center columns per tile, CTA pair
// (0/1), TMA ring stages, candidates kept per frame (8 or 16).
struct TilePlan {
    int bn = 0, pair = 0, stages = 0, list_len = 0;
};
// Every shape that fits for (d, k), widest first.
void tc_enumerate_plans(int d, int k, std::vector<TilePlan> &out);
// While set (nullptr clears), tensor-core calls of this host thread use
// `plan` (and fail with KM_ERR_UNSUPPORTED when it does not fit).
void tc_force_plan(const TilePlan *plan);
// The shape later calls use for (d, k) (km_tune_tiles' choice).
void tc_store_plan(int d, int k, const TilePlan &plan);
void tc_clear_plans();
// The shape a call for (d, k) uses now; *tuned: it comes from the table.
bool tc_current_plan(int d, int k, TilePlan *out, bool *tuned);
size_t tc_frames_ws_size(int64_t n, int d);     // fp16 frame copy + norms
size_t tc_centers_ws_size(int d, int k);        // fp16 centers + norms + shift + scalars
size_t tc_assign_ws_size(int64_t n, int d, int k);  // candidate lists + counters

#define TC_CANDIDATES 16  // candidate centers kept per frame by the tensor-core pass

struct TcBuffers {
    // frames
    void *xh = nullptr;          // n x kp fp16 (centered, scaled; columns d, d+1 = 1)
    float4 *xnorm = nullptr;     // (||x_hat||^2 scaled, bounds of ||x'|| and of its FP16 rounding error, 0)
    // centers
    void *ch = nullptr;          // k_pad x kp fp16 (centered, scaled; columns d, d+1 = -||c_hat||^2/2 hi/lo)
    float2 *cnorm = nullptr;     // bounds of ||c'|| and of its FP16 rounding error per center
    float *shift = nullptr;      // d floats
    uint32_t *scal = nullptr;    // scale, 1/scale^2, norm maxima (float bits)
    // candidate lists
    int32_t *rc_frames = nullptr;           // entry -> frame
    int32_t *pair_center = nullptr;         // pair -> candidate center
    unsigned long long *rc_keys = nullptr;  // entry -> (distance bits, center) minimum
    int32_t *rc_best = nullptr;             // entry -> candidate with the smallest tensor-core distance
    float *pair_lo = nullptr;               // pair -> lower bound of the candidate's exact distance
    int64_t *rc_pairs = nullptr;            // entry -> (first pair << 8) | number of pairs
    int32_t *amb_entries = nullptr;         // entries the FP32 bracket could not settle
    int32_t *amb_mask = nullptr;            // their candidates (bit t: pair first + t) for the exact pass
    int32_t *full_frames = nullptr;
    unsigned long long *full_keys = nullptr;
    int32_t *counters = nullptr;  // [0] recheck entries, [1] full entries, [2] pairs, [3] unsettled entries
    unsigned long long *flipped = nullptr;
    uint32_t *err = nullptr;
    float *chn = nullptr;        // FP8 only: -||c~_j||^2 / 2 per center (the norm is not folded into the GEMM)
    int kp = 0;        // operand row length in elements
    int esize = 2;     // operand bytes per element: 2 (FP16, BF16) or 1 (FP8 e4m3)
    int bf16 = 0;      // operand type of xh / ch: 0 FP16, 1 BF16
    int fp8 = 0;       // 1: e4m3 operands (frames scaled per row), norms applied in the epilogue
    int keep_err = 0;  // 1: tc_assign leaves err as it is (the caller clears it once for several calls)
};

// The same buffers for frames [a, ...): the per-frame arrays start at row a.
inline TcBuffers tc_rows_from(const TcBuffers &b, int64_t a) {
    TcBuffers v = b;
    v.xh = static_cast<char *>(b.xh) + (size_t)a * b.kp * b.esize;
    v.xnorm = b.xnorm + a;
    return v;
}

// Sets the operand type of carved buffers from the precision (KM_PREC_FP16,
// KM_PREC_BF16 or KM_PREC_FP8): element size and row length.
void tc_set_operand(TcBuffers &b, int d, int prec);
void tc_carve_frames(void *ws, int64_t n, int d, TcBuffers &b);
void tc_carve_centers(void *ws, int d, int k, TcBuffers &b);
void tc_carve_assign(void *ws, int64_t n, int d, int k, TcBuffers &b);

// shift == nullptr: the shift is the mean of the centers (computed on device).
int tc_prepare_shift_from_centers(const float *C, int d, int k, TcBuffers &b, cudaStream_t s);
int tc_prepare_frames(const float *X, int64_t n, int d, TcBuffers &b, cudaStream_t s, const PairSrc *ps = nullptr);
int tc_prepare_centers(const float *C, int d, int k, TcBuffers &b, cudaStream_t s);
// Runs the tensor-core pass, the candidate recheck and the full recheck.
// dump (nullable, n x k floats) receives every tensor-core distance;
// wait_cycles (nullable, 8 device counters) the cycles each kernel role
// spent waiting (diagnostics).
int tc_assign(const float *X, int64_t n, int d, const float *C, int k, int32_t *labels,
              TcBuffers &b, cudaStream_t s, ProfEvents *prof = nullptr, float *dump = nullptr,
              unsigned long long *wait_cycles = nullptr, const PairSrc *ps = nullptr);
// The tensor-core pass on s, then the exact re-checks on `side` with their
// changed labels in fl (whose count must be zero when the re-checks start).
// With n_fork > 1 events the pass runs in up to min(n_fork, kTcMaxChunks)
// launches over consecutive frame ranges, each chunk's re-check on `side`
// (after ev_fork[c], recorded on s) beside the next chunk's launch.  labels
// holds the tensor-core labels; the caller joins `side` back into s before
// it applies fl.
constexpr int kTcMaxChunks = 8;
// label_counts (nullable, k ints, zeroed by the caller): the pass adds each
// frame's tensor-core label to it.
int tc_assign_deferred(const float *X, int64_t n, int d, const float *C, int k, int32_t *labels, TcBuffers &b,
                       cudaStream_t s, cudaStream_t side, const cudaEvent_t *ev_fork, int n_fork,
                       const FlipList &fl, ProfEvents *prof = nullptr, const PairSrc *ps = nullptr,
                       int32_t *label_counts = nullptr);

// Resident center sets (capi.cu), used by the serving loop (serve.cu).
int assign_centers_enqueue(const float *X, int64_t n, const km_centers *h, int32_t *labels, void *ws,
                           size_t ws_bytes, uint32_t *err_host, cudaStream_t s);
size_t assign_centers_ws_bytes(int64_t n, const km_centers *h);
int centers_d(const km_centers *h);
// Whether kernels of the current device read host memory (page-locked or
// not) in place through the host's page tables, as on Grace.
bool gpu_reads_host_in_place();
// dst (device) <- src (host memory the device reads in place): a copy kernel
// on s, one small CTA per SM (it fits beside a tensor-core CTA) claiming
// 16 KB blocks from the counter pair ctr (two words, zero before the first
// launch; each launch leaves it zero).  Launches that share ctr must run one
// after the other (one stream).
int launch_host_copy(const float *src, float *dst, int64_t count, unsigned long long *ctr, cudaStream_t s);
int centers_device(const km_centers *h);
int device_error_status(uint32_t e);
// Bits set by km_debug_fake_device_error, cleared as they are taken.
uint32_t take_fake_device_error();

}  // namespace km

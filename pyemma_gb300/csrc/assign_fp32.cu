// assign_fp32.cu -- kernel (a): exact float32 nearest-center assignment on
// the CUDA cores, and kernel (b'): exact re-evaluation of candidate lists.
//
// Reference: ClusterModel(centers, 'euclidean').transform(X) called from
// pyemma/coordinates/clustering/interface.py:157-167.  The distance of frame
// x to center c is sum_f (x_f - c_f)^2 accumulated in float32 in feature
// order with every subtraction, product and sum rounded on its own; the
// label is the lowest index among the minima.
//
// Layout: a CTA of 8 warps owns a tile of 8*FT frames; lanes own centers
// (lane + 32 g, g < G) of a block of 32*G centers.  Frames and centers are
// staged through shared memory in chunks of 32 features with coalesced
// loads; every (frame, center) sum stays in one register in feature order,
// and a lexicographic warp-shuffle (distance, index) reduction finishes the
// argmin.
#include <algorithm>

#include "km_common.cuh"
#include "km_internal.h"

namespace km {

namespace {

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;
constexpr int kFC = 32;  // features per shared-memory chunk

// Full re-check lists of at most this many frames go to full_few_kernel (one
// distance per thread, all in one short wave); longer lists to the tiled
// kernel, which reuses each staged center row for 32 frames.  The choice is
// made on the device from the list's length.
constexpr int64_t kFullFew = 64;

// SPLIT: blockIdx.y selects one block of 32*G centers and the result of the
// block goes to keys[entry] by atomicMin of (distance bits << 32 | center),
// which recheck_finalize_kernel turns into labels.
template <int FT, int G, bool SPLIT>
__global__ void __launch_bounds__(kThreads) assign_fp32_kernel(
    const float *__restrict__ X, const int32_t *__restrict__ frame_idx,
    const int32_t *__restrict__ n_dev, int64_t n_max, int d, const float *__restrict__ C, int k,
    int32_t *__restrict__ labels, float *__restrict__ dist, unsigned long long *flipped,
    unsigned long long *__restrict__ keys) {
    constexpr int BM = kWarps * FT;
    constexpr int BN = 32 * G;
    __shared__ float Xs[BM][kFC];
    __shared__ float Cs[BN][kFC + 1];

    int64_t n = n_max;
    if (n_dev) {
        int64_t nd = *n_dev;
        n = nd < n_max ? nd : n_max;
    }
    if (SPLIT && n <= kFullFew) return;  // full_few_kernel takes short lists
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int64_t ntiles = (n + BM - 1) / BM;
    unsigned long long nflip = 0;

    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t t0 = tile * BM;
        float bd[FT];
        int bj[FT];
#pragma unroll
        for (int t = 0; t < FT; ++t) {
            bd[t] = __int_as_float(0x7f800000);  // +inf
            bj[t] = 0;
        }
        const int cb_begin = SPLIT ? (int)blockIdx.y * BN : 0;
        const int cb_end = SPLIT ? min(k, cb_begin + BN) : k;
        for (int cb = cb_begin; cb < cb_end; cb += BN) {
            float acc[FT][G];
#pragma unroll
            for (int t = 0; t < FT; ++t)
#pragma unroll
                for (int g = 0; g < G; ++g) acc[t][g] = 0.0f;

            for (int fc = 0; fc < d; fc += kFC) {
                const int fw = min(kFC, d - fc);
                __syncthreads();
                for (int e = threadIdx.x; e < BM * fw; e += kThreads) {
                    const int r = e / fw, f = e - r * fw;
                    const int64_t i = t0 + r;
                    float v = 0.0f;
                    if (i < n) {
                        const int64_t row = frame_idx ? (int64_t)frame_idx[i] : i;
                        v = __ldg(X + row * d + fc + f);
                    }
                    Xs[r][f] = v;
                }
                for (int e = threadIdx.x; e < BN * fw; e += kThreads) {
                    const int r = e / fw, f = e - r * fw;
                    const int j = cb + r;
                    Cs[r][f] = j < k ? __ldg(C + (int64_t)j * d + fc + f) : 0.0f;
                }
                __syncthreads();
                for (int f = 0; f < fw; ++f) {
                    float xv[FT], cv[G];
#pragma unroll
                    for (int t = 0; t < FT; ++t) xv[t] = Xs[warp * FT + t][f];
#pragma unroll
                    for (int g = 0; g < G; ++g) cv[g] = Cs[lane + 32 * g][f];
#pragma unroll
                    for (int t = 0; t < FT; ++t)
#pragma unroll
                        for (int g = 0; g < G; ++g) acc[t][g] = __fadd_rn(acc[t][g], sq_term(xv[t], cv[g]));
                }
            }
#pragma unroll
            for (int t = 0; t < FT; ++t)
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    const int j = cb + lane + 32 * g;
                    if (j < k && acc[t][g] < bd[t]) {
                        bd[t] = acc[t][g];
                        bj[t] = j;
                    }
                }
        }
#pragma unroll
        for (int t = 0; t < FT; ++t) {
            warp_argmin(bd[t], bj[t]);
            const int64_t i = t0 + warp * FT + t;
            if (SPLIT) {
                if (lane == 0 && i < n)
                    atomicMin(&keys[i], ((unsigned long long)__float_as_uint(bd[t]) << 32) | (unsigned)bj[t]);
                continue;
            }
            if (lane == 0 && i < n) {
                const int64_t out = frame_idx ? (int64_t)frame_idx[i] : i;
                if (flipped && labels[out] != bj[t]) ++nflip;
                labels[out] = bj[t];
                if (dist) dist[out] = bd[t];
            }
        }
    }
    if (flipped && nflip) atomicAdd(flipped, nflip);
}

template <int FT, int G>
int launch_cfg(const float *X, const int32_t *frame_idx, const int32_t *n_dev, int64_t n, int d,
               const float *C, int k, int32_t *labels, float *dist, unsigned long long *flipped,
               cudaStream_t s) {
    constexpr int BM = kWarps * FT;
    static int per_sm = -1;  // cached: no queries while a stream is being captured
    if (per_sm < 0) {
        int v = 0;
        KM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, assign_fp32_kernel<FT, G, false>, kThreads, 0));
        per_sm = v;
    }
    int64_t ntiles = (n + BM - 1) / BM;
    int64_t grid = (int64_t)num_sms() * (per_sm > 0 ? per_sm : 1);
    if (grid > ntiles) grid = ntiles;
    if (grid < 1) grid = 1;
    assign_fp32_kernel<FT, G, false><<<(unsigned)grid, kThreads, 0, s>>>(X, frame_idx, n_dev, n, d, C, k,
                                                                        labels, dist, flipped, nullptr);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

// Kernel (b'): exact float32 distances of the candidates of re-checked frames.
// A key (distance bits << 32 | center) of a non-negative float orders
// lexicographically as an unsigned integer, so atomicMin keeps the smallest
// distance and, among equal distances, the lowest center.
//
// Phase 1 evaluates, for every entry, the candidate with the smallest
// tensor-core distance.  Phase 2 evaluates the other candidates whose lower
// bound does not exceed that exact distance (the rest can neither win nor
// tie).  One thread per evaluation, sqdist_exact over the two rows: the many
// independent 16-byte loads of each thread keep the memory system busy.
__global__ void __launch_bounds__(256) recheck_best_kernel(
    const float *__restrict__ X, int d, const float *__restrict__ C, const int32_t *__restrict__ rc_frames,
    const int32_t *__restrict__ rc_best, const int32_t *__restrict__ entry_count, int64_t max_entries,
    unsigned long long *__restrict__ keys) {
    int64_t count = *entry_count;
    if (count > max_entries) count = max_entries;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int j = rc_best[e];
        const float dd = sqdist_exact(X + (int64_t)rc_frames[e] * d, C + (int64_t)j * d, d);
        keys[e] = ((unsigned long long)__float_as_uint(dd) << 32) | (unsigned)j;
    }
}

__global__ void __launch_bounds__(256) recheck_rest_kernel(
    const float *__restrict__ X, int d, const float *__restrict__ C, const int32_t *__restrict__ rc_frames,
    const int32_t *__restrict__ rc_best, const int32_t *__restrict__ pair_entry,
    const int32_t *__restrict__ pair_center, const float *__restrict__ pair_lo,
    const int32_t *__restrict__ pair_count, int64_t max_pairs, unsigned long long *__restrict__ keys) {
    int64_t count = *pair_count;
    if (count > max_pairs) count = max_pairs;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < count;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int e = pair_entry[q];
        const int j = pair_center[q];
        if (j == rc_best[e]) continue;
        const float dstar = __uint_as_float((uint32_t)(keys[e] >> 32));
        if (pair_lo[q] > dstar) continue;  // false for NaN: evaluated
        const float dd = sqdist_exact(X + (int64_t)rc_frames[e] * d, C + (int64_t)j * d, d);
        atomicMin(&keys[e], ((unsigned long long)__float_as_uint(dd) << 32) | (unsigned)j);
    }
}

// Full re-check of a short list: one warp per (frame, 32 consecutive
// centers), one exact distance per lane (sqdist_exact: the assignment's
// arithmetic and order), the warp's smallest key, one atomicMin per warp.
__global__ void __launch_bounds__(256) full_few_kernel(const float *__restrict__ X, const int32_t *__restrict__ frames,
                                                       const int32_t *__restrict__ n_dev, int64_t n_max, int d,
                                                       const float *__restrict__ C, int k,
                                                       unsigned long long *__restrict__ keys) {
    int64_t n = *n_dev;
    if (n > n_max) n = n_max;
    if (n > kFullFew) return;  // the tiled kernel takes long lists
    const int lane = threadIdx.x & 31;
    const int64_t groups = (k + 31) / 32;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n * groups; w += nw) {
        const int64_t e = w / groups;
        const int j = (int)((w - e * groups) * 32) + lane;
        unsigned long long key = ~0ull;
        if (j < k) {
            const float dd = sqdist_exact(X + (int64_t)frames[e] * d, C + (int64_t)j * d, d);
            key = ((unsigned long long)__float_as_uint(dd) << 32) | (unsigned)j;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const unsigned long long o = __shfl_xor_sync(0xffffffffu, key, off);
            key = o < key ? o : key;
        }
        if (lane == 0) atomicMin(&keys[e], key);
    }
}

// One thread per entry: the winning key becomes the label (label 0 when no
// candidate distance is finite, as in the exact kernel).  With a flip list
// (flips non-null) a changed label is listed instead of written.
__global__ void __launch_bounds__(256) recheck_finalize_kernel(
    const int32_t *__restrict__ rc_frames, const unsigned long long *__restrict__ keys,
    const int32_t *__restrict__ entry_count, int64_t max_entries, int32_t *__restrict__ labels,
    unsigned long long *flipped, int32_t *__restrict__ flips, int32_t *__restrict__ n_flips, int64_t max_flips) {
    int64_t count = *entry_count;
    if (count > max_entries) count = max_entries;
    unsigned long long nflip = 0;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
         e += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long key = keys[e];
        const uint32_t dbits = (uint32_t)(key >> 32);
        const int lbl = dbits < 0x7f800000u ? (int)(uint32_t)key : 0;
        const int64_t frame = rc_frames[e];
        const int before = labels[frame];
        if (before != lbl) {
            ++nflip;
            if (flips) {
                const int slot = atomicAdd(n_flips, 1);
                if (slot < max_flips) {
                    flips[3 * (int64_t)slot] = (int32_t)frame;
                    flips[3 * (int64_t)slot + 1] = before;
                    flips[3 * (int64_t)slot + 2] = lbl;
                }
            } else {
                labels[frame] = lbl;
            }
        }
    }
    if (flipped && nflip) atomicAdd(flipped, nflip);
}

}  // namespace

int launch_assign_fp32(const float *X, const int32_t *frame_idx, const int32_t *n_dev, int64_t n,
                       int d, const float *C, int k, int32_t *labels, float *dist,
                       unsigned long long *flipped, cudaStream_t s) {
    if (n == 0) return KM_OK;
    if (k <= 32) return launch_cfg<4, 1>(X, frame_idx, n_dev, n, d, C, k, labels, dist, flipped, s);
    if (k <= 64) return launch_cfg<4, 2>(X, frame_idx, n_dev, n, d, C, k, labels, dist, flipped, s);
    if (k <= 128) return launch_cfg<4, 4>(X, frame_idx, n_dev, n, d, C, k, labels, dist, flipped, s);
    // Narrow frames: more frames per thread, so each shared-memory center
    // value feeds more distances (the chunk loop is short at small d).
    if (d <= 32) return launch_cfg<8, 8>(X, frame_idx, n_dev, n, d, C, k, labels, dist, flipped, s);
    return launch_cfg<4, 8>(X, frame_idx, n_dev, n, d, C, k, labels, dist, flipped, s);
}

int launch_recheck_pairs(const float *X, int d, const float *C, const int32_t *rc_frames, const int32_t *rc_best,
                         const int32_t *pair_entry, const int32_t *pair_center, const float *pair_lo,
                         unsigned long long *keys, const int32_t *counters, int64_t max_entries, int64_t max_pairs,
                         int32_t *labels, unsigned long long *flipped, cudaStream_t s, const FlipList *fl,
                         int blocks_per_sm) {
    if (max_entries == 0) return KM_OK;
    const int64_t cap = (int64_t)num_sms() * blocks_per_sm;
    int64_t g0 = (max_entries + 255) / 256;
    if (g0 > cap) g0 = cap;
    recheck_best_kernel<<<(unsigned)(g0 < 1 ? 1 : g0), 256, 0, s>>>(X, d, C, rc_frames, rc_best, counters,
                                                                  max_entries, keys);
    KM_CUDA(cudaGetLastError());
    int64_t g1 = (max_pairs + 255) / 256;
    if (g1 > cap) g1 = cap;
    recheck_rest_kernel<<<(unsigned)(g1 < 1 ? 1 : g1), 256, 0, s>>>(X, d, C, rc_frames, rc_best, pair_entry,
                                                                  pair_center, pair_lo, counters + 2, max_pairs, keys);
    KM_CUDA(cudaGetLastError());
    int64_t g2 = (max_entries + 255) / 256;
    if (g2 > cap) g2 = cap;
    recheck_finalize_kernel<<<(unsigned)(g2 < 1 ? 1 : g2), 256, 0, s>>>(
        rc_frames, keys, counters, max_entries, labels, flipped, fl ? fl->rows : nullptr, fl ? fl->count : nullptr,
        fl ? fl->cap : 0);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

int launch_full_recheck(const float *X, const int32_t *frames, const int32_t *n_dev, int64_t n_max, int d,
                        const float *C, int k, unsigned long long *keys, int32_t *labels,
                        unsigned long long *flipped, cudaStream_t s, const FlipList *fl) {
    if (n_max == 0) return KM_OK;
    // The list is short next to n_max: tiles of 32 frames x 256 centers,
    // one CTA per (frame tile, center block), so that a few thousand frames
    // still occupy every SM.
    constexpr int FT = 4, G = 8, BM = kWarps * FT, BN = 32 * G;
    static int per_sm = -1;
    if (per_sm < 0) {
        int v = 0;
        KM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, assign_fp32_kernel<FT, G, true>, kThreads, 0));
        per_sm = v > 0 ? v : 1;
    }
    const int64_t gy = (k + BN - 1) / BN;
    int64_t gx = (n_max + BM - 1) / BM;
    int64_t cap = (int64_t)num_sms() * per_sm * 2;
    cap = cap / gy > 0 ? cap / gy : 1;
    if (gx > cap) gx = cap;
    if (gy > 65535) {
        set_error("k=%d: too many center blocks for the full re-check", k);
        return KM_ERR_BAD_SHAPE;
    }
    int64_t gf = (std::min(n_max, kFullFew) * ((k + 31) / 32) + 7) / 8;  // 8 warps per block
    const int64_t capf = (int64_t)num_sms() * 8;
    if (gf > capf) gf = capf;
    full_few_kernel<<<(unsigned)(gf < 1 ? 1 : gf), 256, 0, s>>>(X, frames, n_dev, n_max, d, C, k, keys);
    KM_CUDA(cudaGetLastError());
    assign_fp32_kernel<FT, G, true><<<dim3((unsigned)gx, (unsigned)gy), kThreads, 0, s>>>(
        X, frames, n_dev, n_max, d, C, k, nullptr, nullptr, nullptr, keys);
    KM_CUDA(cudaGetLastError());
    int64_t g2 = (n_max + 255) / 256;
    const int64_t cap2 = (int64_t)num_sms() * 8;
    if (g2 > cap2) g2 = cap2;
    recheck_finalize_kernel<<<(unsigned)g2, 256, 0, s>>>(frames, keys, n_dev, n_max, labels, flipped,
                                                          fl ? fl->rows : nullptr, fl ? fl->count : nullptr,
                                                          fl ? fl->cap : 0);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

}  // namespace km

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
#include <type_traits>
#include <cmath>

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
template <int FT, int G, bool SPLIT, class Src>
__global__ void __launch_bounds__(kThreads) assign_fp32_kernel(
    const Src src, const int32_t *__restrict__ frame_idx,
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
                        v = src.get(row, fc + f);
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

template <int FT, int G, class Src>
int launch_cfg(const Src &src, const int32_t *frame_idx, const int32_t *n_dev, int64_t n, int d,
               const float *C, int k, int32_t *labels, float *dist, unsigned long long *flipped,
               cudaStream_t s) {
    constexpr int BM = kWarps * FT;
    static int per_sm_dev[kDeviceSlots] = {};  // per device, cached: no queries while a stream is being captured
    const int dev = current_device();
    int per_sm = dev >= 0 && dev < kDeviceSlots ? per_sm_dev[dev] : 0;
    if (per_sm <= 0) {
        int v = 0;
        KM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, assign_fp32_kernel<FT, G, false, Src>, kThreads, 0));
        per_sm = v > 0 ? v : 1;
        if (dev >= 0 && dev < kDeviceSlots) per_sm_dev[dev] = per_sm;
    }
    int64_t ntiles = (n + BM - 1) / BM;
    int64_t grid = (int64_t)num_sms() * (per_sm > 0 ? per_sm : 1);
    if (grid > ntiles) grid = ntiles;
    if (grid < 1) grid = 1;
    assign_fp32_kernel<FT, G, false, Src><<<(unsigned)grid, kThreads, 0, s>>>(src, frame_idx, n_dev, n, d, C, k,
                                                                             labels, dist, flipped, nullptr);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

// Kernel (b'): the candidates of re-checked frames.
//
// Pass 1 (recheck_fast_kernel), one warp per entry: the float32 squared
// distance F of the frame to each candidate, lanes over the features (16-byte
// loads where rows allow, coalesced), fused multiply-adds and a shuffle tree.
// F differs from the oracle's sequential float32 distance D by a factor
// within [1 - gamma, 1 + gamma] (rounding of the differences, of each lane's
// n_l fused steps and of the 5 tree sums, against D's d + 2 roundings per
// term; gamma = (d + n_l + 10) u, inflated).  With Fu = F (1 + gamma) and
// Fl = F (1 - gamma), a candidate whose Fl exceeds the smallest Fu can
// neither win nor tie.  The candidate with the best tensor-core value goes
// first, and a candidate whose tensor-core lower bound already exceeds the
// smallest Fu so far is not evaluated.  One survivor: the label is settled.
// Several (or a non-finite F): the entry and its survivors go to pass 2.
//
// Pass 2 (recheck_exact_kernel), one thread per surviving candidate:
// sqdist_exact, the assignment's arithmetic and order; the key
// (distance bits << 32 | center) of a non-negative float orders
// lexicographically as an unsigned integer, so atomicMin keeps the smallest
// distance and, among equal distances, the lowest center.  Then
// recheck_finalize_kernel over the pass-2 entries.

// Lane sum of (x - c)^2 over the row pair, lanes over features.
__device__ __forceinline__ float rc_lane_sum(const float *__restrict__ x, const float *__restrict__ c, int d,
                                             bool vec4, int lane);

template <class Src>
__device__ __forceinline__ float rc_lane_sum_src(const Src &src, int64_t i, const float *__restrict__ c, int d,
                                                 bool vec4, int lane) {
    if constexpr (std::is_same<Src, DenseRows>::value) {
        return rc_lane_sum(src.X + i * d, c, d, vec4, lane);
    } else {
        float acc = 0.0f;
        for (int f = lane; f < d; f += 32) {
            const float t = __fsub_rn(src.get(i, f), __ldg(c + f));
            acc = __fmaf_rn(t, t, acc);
        }
        return acc;
    }
}

__device__ __forceinline__ float rc_lane_sum(const float *__restrict__ x, const float *__restrict__ c, int d,
                                             bool vec4, int lane) {
    float acc = 0.0f;
    if (vec4) {
        const float4 *x4 = reinterpret_cast<const float4 *>(x);
        const float4 *c4 = reinterpret_cast<const float4 *>(c);
        for (int f = lane; f < (d >> 2); f += 32) {
            const float4 a = __ldg(x4 + f), b = __ldg(c4 + f);
            float t = __fsub_rn(a.x, b.x);
            acc = __fmaf_rn(t, t, acc);
            t = __fsub_rn(a.y, b.y);
            acc = __fmaf_rn(t, t, acc);
            t = __fsub_rn(a.z, b.z);
            acc = __fmaf_rn(t, t, acc);
            t = __fsub_rn(a.w, b.w);
            acc = __fmaf_rn(t, t, acc);
        }
    } else {
        for (int f = lane; f < d; f += 32) {
            const float t = __fsub_rn(__ldg(x + f), __ldg(c + f));
            acc = __fmaf_rn(t, t, acc);
        }
    }
    return acc;
}

template <class Src>
__global__ void __launch_bounds__(256) recheck_fast_kernel(
    const Src src, int d, const float *__restrict__ C, const int32_t *__restrict__ rc_frames,
    const int32_t *__restrict__ rc_best, const int64_t *__restrict__ rc_pairs, const int32_t *__restrict__ pair_center,
    const float *__restrict__ pair_lo, const int32_t *__restrict__ entry_count, int64_t max_entries, float gamma_lo,
    float gamma_hi, int32_t *__restrict__ labels, unsigned long long *flipped, int32_t *__restrict__ flips,
    int32_t *__restrict__ n_flips, int64_t max_flips, int32_t *__restrict__ amb_entries,
    int32_t *__restrict__ amb_mask, int32_t *__restrict__ amb_count) {
    int64_t count = *entry_count;
    if (count > max_entries) count = max_entries;
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    bool vec4 = (d & 3) == 0 && (reinterpret_cast<uintptr_t>(C) & 15) == 0;
    if constexpr (std::is_same<Src, DenseRows>::value) vec4 = vec4 && (reinterpret_cast<uintptr_t>(src.X) & 15) == 0;
    const float kInf = __int_as_float(0x7f800000);
    unsigned long long nflip = 0;
    for (int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < count; e += nw) {
        const int64_t i = rc_frames[e];
        const int64_t word = rc_pairs[e];
        const int64_t q0 = word >> 8;
        const int m = (int)(word & 0xFF);
        const int jb = rc_best[e];
        // Lane t (< m) holds candidate t's bracket; unevaluated: Fl = +inf.
        float my_fl = kInf;
        bool my_bad = false;
        int my_j = -1;
        if (lane < m) my_j = pair_center[q0 + lane];
        const float my_lo = lane < m ? pair_lo[q0 + lane] : kInf;
        const int tb = __ffs(__ballot_sync(0xffffffffu, lane < m && my_j == jb)) - 1;  // the best tensor-core slot
        float fu_min = kInf;
        for (int k = 0; k < m; ++k) {
            const int t = k == 0 ? (tb >= 0 ? tb : 0) : (k <= tb ? k - 1 : k);
            const float lo_t = __shfl_sync(0xffffffffu, my_lo, t);
            if (lo_t > fu_min) continue;  // cannot win or tie (false for NaN: evaluated)
            const int j = __shfl_sync(0xffffffffu, my_j, t);
            float acc = rc_lane_sum_src(src, i, C + (int64_t)j * d, d, vec4, lane);
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) acc = __fadd_rn(acc, __shfl_xor_sync(0xffffffffu, acc, off));
            const float fu = __fmul_ru(acc, gamma_hi);
            const float fl = __fmul_rd(acc, gamma_lo);
            if (lane == t) {
                my_fl = fl;
                my_bad = !(acc <= 3.4028234663852886e38f);  // NaN or infinite
            }
            if (fu < fu_min) fu_min = fu;
        }
        const bool any_bad = __any_sync(0xffffffffu, my_bad);
        const unsigned alive = __ballot_sync(0xffffffffu, lane < m && (any_bad ? my_fl < kInf || my_bad : my_fl <= fu_min));
        if (!any_bad && __popc(alive) == 1) {
            const int t = __ffs(alive) - 1;
            const int lbl = __shfl_sync(0xffffffffu, my_j, t);
            if (lane == 0) {
                const int before = labels[i];
                if (before != lbl) {
                    ++nflip;
                    if (flips) {
                        const int slot = atomicAdd(n_flips, 1);
                        if (slot < max_flips) {
                            flips[3 * (int64_t)slot] = (int32_t)i;
                            flips[3 * (int64_t)slot + 1] = before;
                            flips[3 * (int64_t)slot + 2] = lbl;
                        }
                    } else {
                        labels[i] = lbl;
                    }
                }
            }
        } else if (lane == 0) {
            // every evaluated candidate when some F is not finite
            const int slot = atomicAdd(amb_count, 1);
            amb_entries[slot] = (int32_t)e;
            amb_mask[slot] = (int32_t)alive;
        }
    }
    if (flipped && lane == 0 && nflip) atomicAdd(flipped, nflip);
}

// The exact float32 distance of one row pair by a whole warp: lanes load and
// square 32 features at a time (coalesced), and the 32 squares go to every
// lane in feature order by shuffles, so each lane adds them in the oracle's
// sequence: the result is sqdist_exact's, bit for bit, in every lane.  One
// thread walking the row waits on memory for every group of loads; here the
// wait is shared by 32 lanes.
template <class Src>
__device__ __forceinline__ float warp_sqdist_exact(const Src &src, int64_t i, const float *__restrict__ c, int d,
                                                   int lane) {
    float acc = 0.0f;
    for (int f0 = 0; f0 < d; f0 += 32) {
        const int f = f0 + lane;
        const float q = f < d ? sq_term(src.get(i, f), __ldg(c + f)) : 0.0f;
        const int fw = min(32, d - f0);
        if (fw == 32) {
#pragma unroll
            for (int l = 0; l < 32; ++l) acc = __fadd_rn(acc, __shfl_sync(0xffffffffu, q, l));
        } else {
            for (int l = 0; l < fw; ++l) acc = __fadd_rn(acc, __shfl_sync(0xffffffffu, q, l));
        }
    }
    return acc;
}

// Pass 2, one warp per (unsettled entry, candidate slot); slots outside the
// entry's mask are skipped.
template <class Src>
__global__ void __launch_bounds__(256) recheck_exact_kernel(
    const Src src, int d, const float *__restrict__ C, const int32_t *__restrict__ rc_frames,
    const int64_t *__restrict__ rc_pairs, const int32_t *__restrict__ pair_center,
    const int32_t *__restrict__ amb_entries, const int32_t *__restrict__ amb_mask,
    const int32_t *__restrict__ amb_count, int64_t max_entries, unsigned long long *__restrict__ keys) {
    int64_t count = *amb_count;
    if (count > max_entries) count = max_entries;
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < count * 16; w += nw) {
        const int64_t s = w >> 4;
        const int t = (int)(w & 15);
        if (!((amb_mask[s] >> t) & 1)) continue;
        const int e = amb_entries[s];
        const int j = pair_center[(rc_pairs[e] >> 8) + t];
        const float dd = warp_sqdist_exact(src, (int64_t)rc_frames[e], C + (int64_t)j * d, d, lane);
        if (lane == 0) atomicMin(&keys[e], ((unsigned long long)__float_as_uint(dd) << 32) | (unsigned)j);
    }
}

// Full re-check of a short list: one warp per (frame, center), the exact
// distance by warp_sqdist_exact, one atomicMin per warp.
template <class Src>
__global__ void __launch_bounds__(256) full_few_kernel(const Src src, const int32_t *__restrict__ frames,
                                                       const int32_t *__restrict__ n_dev, int64_t n_max, int d,
                                                       const float *__restrict__ C, int k,
                                                       unsigned long long *__restrict__ keys) {
    int64_t n = *n_dev;
    if (n > n_max) n = n_max;
    if (n > kFullFew) return;  // the tiled kernel takes long lists
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n * k; w += nw) {
        const int64_t e = w / k;
        const int j = (int)(w - e * k);
        const float dd = warp_sqdist_exact(src, (int64_t)frames[e], C + (int64_t)j * d, d, lane);
        if (lane == 0) atomicMin(&keys[e], ((unsigned long long)__float_as_uint(dd) << 32) | (unsigned)j);
    }
}

// One thread per entry (entries[s] with an entry list, else s): the winning
// key becomes the label (label 0 when no candidate distance is finite, as in
// the exact kernel).  With a flip list (flips non-null) a changed label is
// listed instead of written.
__global__ void __launch_bounds__(256) recheck_finalize_kernel(
    const int32_t *__restrict__ rc_frames, const unsigned long long *__restrict__ keys,
    const int32_t *__restrict__ entries, const int32_t *__restrict__ entry_count, int64_t max_entries,
    int32_t *__restrict__ labels, unsigned long long *flipped, int32_t *__restrict__ flips,
    int32_t *__restrict__ n_flips, int64_t max_flips) {
    int64_t count = *entry_count;
    if (count > max_entries) count = max_entries;
    unsigned long long nflip = 0;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < count;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = entries ? entries[s] : s;
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

namespace {

template <class Src>
int assign_fp32_src(const Src &src, const int32_t *frame_idx, const int32_t *n_dev, int64_t n, int d, const float *C,
                    int k, int32_t *labels, float *dist, unsigned long long *flipped, cudaStream_t s) {
    if (k <= 32) return launch_cfg<4, 1>(src, frame_idx, n_dev, n, d, C, k, labels, dist, flipped, s);
    if (k <= 64) return launch_cfg<4, 2>(src, frame_idx, n_dev, n, d, C, k, labels, dist, flipped, s);
    if (k <= 128) return launch_cfg<4, 4>(src, frame_idx, n_dev, n, d, C, k, labels, dist, flipped, s);
    // Narrow frames: more frames per thread, so each shared-memory center
    // value feeds more distances (the chunk loop is short at small d).
    if (d <= 32) return launch_cfg<8, 8>(src, frame_idx, n_dev, n, d, C, k, labels, dist, flipped, s);
    return launch_cfg<4, 8>(src, frame_idx, n_dev, n, d, C, k, labels, dist, flipped, s);
}

template <class Src>
int recheck_pairs_src(const Src &src, int d, const float *C, const int32_t *rc_frames, const int32_t *rc_best,
                      const int64_t *rc_pairs, const int32_t *pair_center, const float *pair_lo,
                      unsigned long long *keys, int32_t *amb_entries, int32_t *amb_mask, int32_t *counters,
                      int64_t max_entries, int32_t *labels, unsigned long long *flipped, cudaStream_t s,
                      const FlipList *fl, int blocks_per_sm) {
    const int64_t cap = (int64_t)num_sms() * blocks_per_sm;
    // gamma = (d + n_l + 10) u, n_l = the largest number of fused steps a
    // lane makes (ceil(d/32), or 4 ceil(d/128) with 16-byte loads), inflated
    // by 1%; the factors are rounded outwards.
    const double u = std::ldexp(1.0, -24);
    const int n_l = std::max((d + 31) / 32, 4 * ((d + 127) / 128));
    const double gamma = (d + n_l + 10) * u * 1.01;
    const float g_lo = std::nextafter((float)(1.0 - gamma), 0.0f);
    const float g_hi = std::nextafter((float)(1.0 + gamma), 2.0f);
    int64_t g0 = (max_entries * 32 + 255) / 256;
    if (g0 > cap) g0 = cap;
    recheck_fast_kernel<Src><<<(unsigned)(g0 < 1 ? 1 : g0), 256, 0, s>>>(
        src, d, C, rc_frames, rc_best, rc_pairs, pair_center, pair_lo, counters, max_entries, g_lo, g_hi, labels,
        flipped, fl ? fl->rows : nullptr, fl ? fl->count : nullptr, fl ? fl->cap : 0, amb_entries, amb_mask,
        counters + 3);
    KM_CUDA(cudaGetLastError());
    int64_t g1 = (max_entries * 16 * 32 + 255) / 256;  // a warp per (entry, slot)
    if (g1 > cap) g1 = cap;
    recheck_exact_kernel<Src><<<(unsigned)(g1 < 1 ? 1 : g1), 256, 0, s>>>(
        src, d, C, rc_frames, rc_pairs, pair_center, amb_entries, amb_mask, counters + 3, max_entries, keys);
    KM_CUDA(cudaGetLastError());
    int64_t g2 = (max_entries + 255) / 256;  // the unsettled list is short: one CTA per SM at most
    if (g2 > num_sms()) g2 = num_sms();
    recheck_finalize_kernel<<<(unsigned)(g2 < 1 ? 1 : g2), 256, 0, s>>>(
        rc_frames, keys, amb_entries, counters + 3, max_entries, labels, flipped, fl ? fl->rows : nullptr,
        fl ? fl->count : nullptr, fl ? fl->cap : 0);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

template <class Src>
int full_recheck_src(const Src &src, const int32_t *frames, const int32_t *n_dev, int64_t n_max, int d,
                     const float *C, int k, unsigned long long *keys, int32_t *labels, unsigned long long *flipped,
                     cudaStream_t s, const FlipList *fl) {
    // Tiles of 32 frames x 256 centers, one CTA per (frame tile, center
    // block).  The list is usually empty or short (full_few_kernel takes up
    // to kFullFew frames and this kernel then exits at once); the grid walks
    // the frame tiles, two CTAs per SM in all.
    constexpr int FT = 4, G = 8, BM = kWarps * FT, BN = 32 * G;
    const int64_t gy = (k + BN - 1) / BN;
    int64_t gx = (n_max + BM - 1) / BM;
    int64_t cap = (int64_t)num_sms() * 2;
    cap = cap / gy > 0 ? cap / gy : 1;
    if (gx > cap) gx = cap;
    if (gy > 65535) {
        set_error("k=%d: too many center blocks for the full re-check", k);
        return KM_ERR_BAD_SHAPE;
    }
    int64_t gf = (std::min(n_max, kFullFew) * k + 7) / 8;  // a warp per (frame, center), 8 warps per block
    const int64_t capf = (int64_t)num_sms() * 4;
    if (gf > capf) gf = capf;
    full_few_kernel<Src><<<(unsigned)(gf < 1 ? 1 : gf), 256, 0, s>>>(src, frames, n_dev, n_max, d, C, k, keys);
    KM_CUDA(cudaGetLastError());
    assign_fp32_kernel<FT, G, true, Src><<<dim3((unsigned)gx, (unsigned)gy), kThreads, 0, s>>>(
        src, frames, n_dev, n_max, d, C, k, nullptr, nullptr, nullptr, keys);
    KM_CUDA(cudaGetLastError());
    int64_t g2 = (n_max + 255) / 256;
    const int64_t cap2 = (int64_t)num_sms();
    if (g2 > cap2) g2 = cap2;
    recheck_finalize_kernel<<<(unsigned)g2, 256, 0, s>>>(frames, keys, nullptr, n_dev, n_max, labels, flipped,
                                                          fl ? fl->rows : nullptr, fl ? fl->count : nullptr,
                                                          fl ? fl->cap : 0);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

PairRows pair_rows(const PairSrc &ps, int d) {
    return PairRows{ps.xyz, reinterpret_cast<const int2 *>(ps.pairs), ps.n_atoms, d};
}

}  // namespace

int launch_assign_fp32(const float *X, const int32_t *frame_idx, const int32_t *n_dev, int64_t n,
                       int d, const float *C, int k, int32_t *labels, float *dist,
                       unsigned long long *flipped, cudaStream_t s, const PairSrc *ps) {
    if (n == 0) return KM_OK;
    if (ps) return assign_fp32_src(pair_rows(*ps, d), frame_idx, n_dev, n, d, C, k, labels, dist, flipped, s);
    return assign_fp32_src(DenseRows{X, d}, frame_idx, n_dev, n, d, C, k, labels, dist, flipped, s);
}

int launch_recheck_pairs(const float *X, int d, const float *C, const int32_t *rc_frames, const int32_t *rc_best,
                         const int64_t *rc_pairs, const int32_t *pair_center, const float *pair_lo,
                         unsigned long long *keys, int32_t *amb_entries, int32_t *amb_mask, int32_t *counters,
                         int64_t max_entries, int32_t *labels, unsigned long long *flipped, cudaStream_t s,
                         const FlipList *fl, int blocks_per_sm, const PairSrc *ps) {
    if (max_entries == 0) return KM_OK;
    if (ps)
        return recheck_pairs_src(pair_rows(*ps, d), d, C, rc_frames, rc_best, rc_pairs, pair_center, pair_lo, keys,
                                 amb_entries, amb_mask, counters, max_entries, labels, flipped, s, fl, blocks_per_sm);
    return recheck_pairs_src(DenseRows{X, d}, d, C, rc_frames, rc_best, rc_pairs, pair_center, pair_lo, keys,
                             amb_entries, amb_mask, counters, max_entries, labels, flipped, s, fl, blocks_per_sm);
}

int launch_full_recheck(const float *X, const int32_t *frames, const int32_t *n_dev, int64_t n_max, int d,
                        const float *C, int k, unsigned long long *keys, int32_t *labels,
                        unsigned long long *flipped, cudaStream_t s, const FlipList *fl, const PairSrc *ps) {
    if (n_max == 0) return KM_OK;
    if (ps) return full_recheck_src(pair_rows(*ps, d), frames, n_dev, n_max, d, C, k, keys, labels, flipped, s, fl);
    return full_recheck_src(DenseRows{X, d}, frames, n_dev, n_max, d, C, k, keys, labels, flipped, s, fl);
}

}  // namespace km

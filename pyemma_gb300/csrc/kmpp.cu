// kmpp.cu -- kernel (d): kmeans++ D^2 sampling.
//
// Reference: KMeans(init_strategy='kmeans++', fixed_seed=seed).fit, called at
// pyemma/coordinates/clustering/kmeans.py:211-212,253 (seed rules at
// kmeans.py:146-164).  The first center is a uniformly drawn frame; every
// later center is drawn with probability proportional to D^2(x), the squared
// distance of x to the nearest center chosen so far.
//
// Determinism: D^2 is the exact float32 distance of the assignment kernel.
// Weights are quantised once per run to integers w_i = floor(D^2_i * 2^e)
// with e fixed after the first round so that the sum of all weights stays
// below 2^62; every sum and prefix sum is then exact, so the draw does not
// depend on the reduction order.  Round r draws a 64-bit number u from
// Philox4x32-10 (counter (r, 0, tag, 0), key (seed, tag)), takes
// t = floor(u * W / 2^64) for the weight total W and picks the first frame
// whose inclusive prefix weight exceeds t.
//
// Per round one launch: a pass over X (distance to the newest center,
// running minimum, per-tile weight sums; HBM-bound), after which the CTA that
// finishes last (a fenced atomic count, no waiting) draws the round's frame
// and copies it into the centers.
//
// Pruning (Euclidean metric, large n d): each frame keeps, besides
// D^2 = mind, the index a of a center whose exact distance is mind.  Round r
// (r >= 2) runs three launches:
//   1. cc_j = ||c_new - c_j||^2 for every earlier center j (float32);
//   2. a pass over (mind, a) only: by the triangle inequality
//      ||x - c_new|| >= ||c_new - c_a|| - ||x - c_a||, so when cc_a >= 4 mind
//      (times a factor covering the float32 rounding of mind, of the new
//      distance and of cc) the exact new distance cannot fall below mind;
//      the other frames go into a list;
//   3. the listed frames' exact distances, spread over every SM; a frame
//      whose minimum drops updates mind and a, and adds the change of its
//      integer weight to its tile's sum; the CTA that finishes last draws.
// The running minima, and so the draws, are the same as without pruning, bit
// for bit.  A skipped frame costs 8 bytes (mind, a) instead of 4d + 4, and
// the tile sums are kept exact by the integer deltas (the first round stores
// them in full).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <type_traits>

#include "km_common.cuh"
#include "km_internal.h"
#include "km_rmsd.cuh"

namespace km {

namespace {

constexpr int kTile = 2048;  // frames per weight tile
constexpr int kTileThreads = 256;

struct KmppWs {
    float *mind;
    int32_t *near;  // a center whose exact distance is mind (pruned Euclidean pass)
    float *cc;      // bounds of ||c_new - c_j||^2 for the current round
    unsigned long long *tile_sum;
    uint32_t *maxbits;
    int *qexp;      // e of the weights floor(D^2 2^e); INT_MIN: every weight is 0
    unsigned int *done;  // CTAs of the current round that have finished
    int32_t *list;       // frames of the round that the bound does not rule out
    int32_t *list_n;
};

KmppWs carve(void *ws, int64_t n, int k, size_t *bytes) {
    Carver c(ws);
    KmppWs w;
    const int64_t ntiles = (n + kTile - 1) / kTile;
    w.mind = c.take<float>(n > 0 ? n : 1);
    w.near = c.take<int32_t>(n > 0 ? n : 1);
    w.cc = c.take<float>(k > 0 ? k : 1);
    w.tile_sum = c.take<unsigned long long>(ntiles > 0 ? ntiles : 1);
    w.maxbits = c.take<uint32_t>(1);
    w.qexp = c.take<int>(1);
    w.done = c.take<unsigned int>(1);
    w.list = c.take<int32_t>(n > 0 ? n : 1);
    w.list_n = c.take<int32_t>(1);
    if (bytes) *bytes = c.bytes();
    return w;
}

// floor(w 2^e) for a finite w > 0, else 0: the integer weight of a squared
// distance, from the float's bits (no FP64 arithmetic; equal to converting
// the exact double product w * 2^e).  e is chosen so that every weight fits.
__device__ __forceinline__ unsigned long long quant_weight(float w, int e) {
    const uint32_t b = __float_as_uint(w);
    if (e == INT_MIN || b == 0u || b >= 0x7f800000u) return 0ull;  // also every negative value
    const int be = (int)(b >> 23);
    const unsigned long long m = be ? (unsigned long long)((b & 0x7FFFFFu) | 0x800000u) : (unsigned long long)b;
    const int sh = (be ? be : 1) - 150 + e;
    if (sh >= 0) return m << sh;
    return sh <= -32 ? 0ull : (m >> (-sh));
}

__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long v,
                                                            unsigned long long *red) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    unsigned long long s = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    return s;  // valid in thread 0
}

// D^2 of frame i to center c (round r's newest center, frame idx[r] under
// the minRMSD metric).
__device__ __forceinline__ float kmpp_d2(const float *__restrict__ X, int64_t i, int d, const float *__restrict__ c,
                                         const KmppMetric &m, int r) {
    if (!m.Xc) return sqdist_exact(X + i * d, c, d);
    const int64_t p = m.idx[r];
    return __double2float_rn(rmsd_msd_rows(m.Xc + i * d, m.Xc + p * d, m.G[i], m.G[p], d / 3));
}

// The exact float32 D^2 of frame i of a row source to the center c.
template <class Src>
__device__ __forceinline__ float src_d2(const Src &src, int64_t i, const float *__restrict__ c, int d) {
    if constexpr (std::is_same<Src, DenseRows>::value)
        return sqdist_exact(src.X + i * d, c, d);
    else
        return sqdist_exact_src(src, i, c, d);
}

// Round 1 pass: mind = D^2 to center 0 (near = 0); max of the finite values.
template <class Src>
__global__ void __launch_bounds__(kTileThreads) kmpp_first_kernel(
    const Src src, int64_t n, int d, const float *__restrict__ c0,
    float *__restrict__ mind, int32_t *__restrict__ near, uint32_t *__restrict__ maxbits, KmppMetric m) {
    float mx = 0.0f;
    const int64_t t0 = (int64_t)blockIdx.x * kTile;
    for (int u = 0; u < kTile / kTileThreads; ++u) {
        const int64_t i = t0 + u * kTileThreads + threadIdx.x;
        if (i < n) {
            float dd;
            if constexpr (std::is_same<Src, DenseRows>::value)
                dd = kmpp_d2(src.X, i, d, c0, m, 0);
            else
                dd = src_d2(src, i, c0, d);
            mind[i] = dd;
            near[i] = 0;
            if (dd < __int_as_float(0x7f800000) && dd > mx) mx = dd;
        }
    }
    for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    if ((threadIdx.x & 31) == 0 && mx > 0.0f) atomicMax(maxbits, __float_as_uint(mx));
}

// e = 62 - ceil(log2 n) - E(max) with 2^(E-1) <= max < 2^E (weights
// floor(D^2 2^e)); INT_MIN when no distance is finite and positive.
__global__ void kmpp_scale_kernel(const uint32_t *__restrict__ maxbits, int64_t n, int *__restrict__ qexp) {
    const uint32_t b = *maxbits;
    const float m = __uint_as_float(b);
    if (!(m > 0.0f) || m == __int_as_float(0x7f800000)) {
        *qexp = INT_MIN;
        return;
    }
    int L = 0;
    while ((int64_t(1) << L) < n) ++L;
    const int be = (int)((b >> 23) & 0xFFu);
    int E;
    if (be) {
        E = be - 126;
    } else {
        const int p = 31 - __clz(b & 0x7FFFFFu);
        E = p - 148;
    }
    *qexp = 62 - L - E;
}

// Round r's bounds: cc[j] = the float32 value of ||C0[rc] - C0[j]||^2 for
// j < rc, one warp per center (lanes stride over the features with fused
// multiply-adds, then a shuffle tree).  Its rounding is covered by the prune
// factor (prune_factor()).
__global__ void __launch_bounds__(256) kmpp_cc_kernel(const float *__restrict__ C0, int d, int rc,
                                                      float *__restrict__ cc) {
    const int j = (int)(blockIdx.x * 8 + (threadIdx.x >> 5));
    const int lane = threadIdx.x & 31;
    if (j >= rc) return;
    const float *a = C0 + (int64_t)rc * d;
    const float *b = C0 + (int64_t)j * d;
    float acc = 0.0f;
    for (int f = lane; f < d; f += 32) {
        const float t = __fsub_rn(__ldg(a + f), __ldg(b + f));
        acc = __fmaf_rn(t, t, acc);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc = __fadd_rn(acc, __shfl_xor_sync(0xffffffffu, acc, off));
    if (lane == 0) cc[j] = acc;
}

// Exclusive prefix sum of v over the CTA (THREADS threads, warp shuffles
// and one pass over the warp totals); *total gets the sum.
template <int THREADS>
__device__ __forceinline__ unsigned long long cta_exclusive_scan_u64(unsigned long long v,
                                                                     unsigned long long *warp_tot,
                                                                     unsigned long long *total) {
    constexpr int kWarps = THREADS / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    __syncthreads();  // warp_tot of an earlier scan has been read
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < kWarps ? warp_tot[lane] : 0ull;
#pragma unroll
        for (int off = 1; off < kWarps; off <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += y;
        }
        if (lane < kWarps) warp_tot[lane] = w;
    }
    __syncthreads();
    *total = warp_tot[kWarps - 1];
    return (warp > 0 ? warp_tot[warp - 1] : 0ull) + x - v;
}

// The draw of round r by the CTA that finished last (the tile sums and the
// minima of the other CTAs are read past L1): t = floor(u W / 2^64) for the
// weight total W over the ntiles tiles, the first frame whose inclusive
// prefix weight exceeds t (a uniform frame when W = 0), copied into C0[r].
template <int THREADS, class Src>
__device__ __forceinline__ void kmpp_draw_round(int64_t ntiles, const Src &src, int64_t n, int d,
                                                float *__restrict__ C0, int64_t *__restrict__ idx_out,
                                                const float *__restrict__ mind, int qexp,
                                                const unsigned long long *__restrict__ tile_sum,
                                                unsigned int *__restrict__ done, int r, uint32_t seed) {
    constexpr int kPer = kTile / THREADS;  // frames per thread in the draw's tile
    __shared__ unsigned long long red[THREADS / 32];
    __shared__ long long tile_hit, pick;
    __shared__ unsigned long long target;
    if (threadIdx.x == 0) {
        tile_hit = -1;
        pick = -1;
    }
    __syncthreads();
    const uint64_t u = kmpp_draw(seed, (uint32_t)r);
    const int64_t per = (ntiles + THREADS - 1) / THREADS;
    const int64_t lo = min((int64_t)threadIdx.x * per, ntiles), hi = min(lo + per, ntiles);
    unsigned long long ts = 0;
    for (int64_t b = lo; b < hi; ++b) ts += __ldcg(tile_sum + b);
    unsigned long long total;
    const unsigned long long excl = cta_exclusive_scan_u64<THREADS>(ts, red, &total);
    if (total > 0) {
        const unsigned long long t = __umul64hi(u, total);
        if (excl <= t && t < excl + ts) {
            unsigned long long run = excl;
            for (int64_t b = lo; b < hi; ++b) {
                const unsigned long long w = __ldcg(tile_sum + b);
                if (t < run + w) {
                    tile_hit = b;
                    target = t - run;
                    break;
                }
                run += w;
            }
        }
    }
    __syncthreads();
    if (tile_hit >= 0) {
        // Inside the tile: kPer consecutive frames per thread.
        const int64_t f0 = tile_hit * kTile + (int64_t)threadIdx.x * kPer;
        unsigned long long w[kPer], ws = 0;
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            w[q] = f0 + q < n ? quant_weight(__ldcg(mind + f0 + q), qexp) : 0ull;
            ws += w[q];
        }
        unsigned long long tile_total;
        unsigned long long run = cta_exclusive_scan_u64<THREADS>(ws, red, &tile_total);
        const unsigned long long tt = target;
        if (run <= tt && tt < run + ws) {
#pragma unroll
            for (int q = 0; q < kPer; ++q) {
                if (tt < run + w[q]) {
                    pick = f0 + q;
                    break;
                }
                run += w[q];
            }
        }
    }
    __syncthreads();
    if (pick < 0 && threadIdx.x == 0) pick = (long long)__umul64hi(u, (unsigned long long)n);
    __syncthreads();
    const int64_t p = pick;
    for (int f = threadIdx.x; f < d; f += THREADS) C0[(int64_t)r * d + f] = src.get(p, f);
    if (threadIdx.x == 0) {
        if (idx_out) idx_out[r] = p;
        *done = 0u;  // for the next round's launch
    }
}

// True in every thread of the CTA that counts itself last among gridDim.x
// (after a fence of this thread's writes); the others' writes are visible
// to it past L1.
__device__ __forceinline__ bool kmpp_last_cta(unsigned int *__restrict__ done) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// Round r >= 1, one CTA per tile of kTile frames, one thread per frame (at
// a time).  With r_center >= 0 the running minimum first takes the distance
// to center r_center (rounds >= 2; round 1 uses the minimum of
// kmpp_first_kernel as it is).  Then the tile's weight sum is stored and the
// CTA that finishes last draws.  THREADS = 1024 for the Euclidean metric
// (two frames per thread: the pass is latency-bound at small n), 256 for
// minRMSD (the QCP solve needs the registers).  The pruned rounds' first
// round runs here too (r_center = -1), which stores every tile sum.
template <int THREADS, bool RMSD, class Src>
__global__ void __launch_bounds__(THREADS) kmpp_round_kernel(
    const Src src, int64_t n, int d, float *__restrict__ C0, int64_t *__restrict__ idx_out,
    float *__restrict__ mind, const int *__restrict__ qexp_p, unsigned long long *__restrict__ tile_sum,
    unsigned int *__restrict__ done, KmppMetric m, int r_center, int r, uint32_t seed) {
    constexpr int kPer = kTile / THREADS;
    __shared__ unsigned long long red[THREADS / 32];
    const int qexp = *qexp_p;
    const int64_t t0 = (int64_t)blockIdx.x * kTile;
    unsigned long long s = 0;
    for (int u = 0; u < kPer; ++u) {
        const int64_t i = t0 + u * THREADS + threadIdx.x;
        if (i < n) {
            float mi = mind[i];
            if (r_center >= 0) {
                const float *c = C0 + (int64_t)r_center * d;
                float dd;
                if constexpr (RMSD)
                    dd = kmpp_d2(src.X, i, d, c, m, r_center);
                else
                    dd = src_d2(src, i, c, d);
                if (dd < mi) {
                    mi = dd;
                    mind[i] = mi;
                }
            }
            s += quant_weight(mi, qexp);
        }
    }
    s = block_sum_u64(s, red);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = s;
    if (!kmpp_last_cta(done)) return;
    kmpp_draw_round<THREADS>(gridDim.x, src, n, d, C0, idx_out, mind, qexp, tile_sum, done, r, seed);
}

// Pruned round, launch 2: four frames per thread (vector loads of mind and
// a); the frames that the bound does not rule out are appended to the list,
// one atomic per warp.  The skip needs a finite mind; a NaN bound never
// skips.
__global__ void __launch_bounds__(256) kmpp_prune_kernel(int64_t n, const float *__restrict__ mind,
                                                         const int32_t *__restrict__ near,
                                                         const float *__restrict__ cc, float prune_factor,
                                                         int32_t *__restrict__ list, int32_t *__restrict__ list_n) {
    const int lane = threadIdx.x & 31;
    const int64_t nq = (n + 3) / 4;
    for (int64_t q0 = (int64_t)blockIdx.x * blockDim.x; q0 < nq; q0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = q0 + threadIdx.x;
        float mi[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        int32_t a[4] = {0, 0, 0, 0};
        const int64_t i0 = 4 * q;
        if (i0 + 3 < n) {
            const float4 m4 = __ldg(reinterpret_cast<const float4 *>(mind) + q);
            const int4 a4 = __ldg(reinterpret_cast<const int4 *>(near) + q);
            mi[0] = m4.x, mi[1] = m4.y, mi[2] = m4.z, mi[3] = m4.w;
            a[0] = a4.x, a[1] = a4.y, a[2] = a4.z, a[3] = a4.w;
        } else {
            for (int v = 0; v < 4; ++v)
                if (i0 + v < n) {
                    mi[v] = mind[i0 + v];
                    a[v] = near[i0 + v];
                }
        }
        unsigned keep = 0u;
#pragma unroll
        for (int v = 0; v < 4; ++v)
            if (i0 + v < n && !(mi[v] <= 3.4028234663852886e38f && __ldg(cc + a[v]) >= __fmul_ru(mi[v], prune_factor)))
                keep |= 1u << v;
        const int cnt = __popc(keep);
        int excl = cnt;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, excl, off);
            if (lane >= off) excl += y;
        }
        const int total = __shfl_sync(0xffffffffu, excl, 31);
        int base = 0;
        if (lane == 31 && total > 0) base = atomicAdd(list_n, total);
        base = __shfl_sync(0xffffffffu, base, 31) + excl - cnt;
        for (int v = 0; v < 4; ++v)
            if ((keep >> v) & 1u) list[base++] = (int32_t)(i0 + v);
    }
}

// Pruned round, launch 3: the listed frames' exact distances, 32 frames per
// warp at a time (grid-stride over the groups of 32 list entries; rows of
// fewer than 32 features take one frame per thread instead).  For
// each run of 32 features, lane f holds feature f0 + f of one listed frame
// at a time (stored rows: one coalesced 128-byte load per frame, where a
// thread per frame makes every load touch 32 rows), squares its difference
// to the center and stores it transposed in shared memory; lane j then adds
// frame j's 32 squares in feature order.  So each distance is the same
// sequence of float32 operations as sqdist_exact (every subtraction, square
// and addition rounded once, features in order), bit for bit.  A smaller
// distance replaces mind and a and moves the frame's integer weight in its
// tile's sum (modular 64-bit deltas, exact).  The CTA that finishes last
// clears the list and draws.
constexpr int kEvalWarps = 8;

template <class Src>
__global__ void __launch_bounds__(kEvalWarps * 32) kmpp_eval_kernel(
    const Src src, int64_t n, int d, float *__restrict__ C0, int64_t *__restrict__ idx_out,
    float *__restrict__ mind, int32_t *__restrict__ near, const int *__restrict__ qexp_p,
    unsigned long long *__restrict__ tile_sum, unsigned int *__restrict__ done, const int32_t *__restrict__ list,
    int32_t *__restrict__ list_n, int64_t ntiles, int r_center, int r, uint32_t seed) {
    __shared__ float sq_s[kEvalWarps][32][33];  // [feature][frame], padded: conflict-free both ways
    __shared__ int32_t frame_s[kEvalWarps][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float(*sq)[33] = sq_s[warp];
    int32_t *frames = frame_s[warp];
    const int qexp = *qexp_p;
    const int64_t cnt = *list_n;
    const float *c = C0 + (int64_t)r_center * d;
    // A smaller distance dd of frame i replaces mind and a, and moves the
    // frame's integer weight in its tile's sum.
    auto lower = [&](int64_t i, float dd) {
        const float mi = mind[i];
        if (dd < mi) {
            mind[i] = dd;
            near[i] = r_center;
            const unsigned long long delta = quant_weight(dd, qexp) - quant_weight(mi, qexp);
            if (delta) atomicAdd(&tile_sum[i / kTile], delta);
        }
    };
    if (d < 32) {
        // Rows shorter than a warp: one frame per thread.
        for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < cnt;
             e += (int64_t)gridDim.x * blockDim.x) {
            const int64_t i = list[e];
            lower(i, src_d2(src, i, c, d));
        }
    } else {
        const int64_t groups = (cnt + 31) / 32;
        for (int64_t g = (int64_t)blockIdx.x * kEvalWarps + warp; g < groups;
             g += (int64_t)gridDim.x * kEvalWarps) {
            const int m = (int)(cnt - g * 32 < 32 ? cnt - g * 32 : 32);  // frames in this group
            const int32_t mine = lane < m ? list[g * 32 + lane] : 0;
            frames[lane] = mine;
            __syncwarp();
            float acc = 0.0f;
            for (int f0 = 0; f0 < d; f0 += 32) {
                const int f = f0 + lane;
                const bool in = f < d;
                const float cf = in ? __ldg(c + f) : 0.0f;
                float v[32];
#pragma unroll
                for (int j = 0; j < 32; ++j) v[j] = (j < m && in) ? src.get(frames[j], f) : 0.0f;
#pragma unroll
                for (int j = 0; j < 32; ++j) sq[lane][j] = sq_term(v[j], cf);
                __syncwarp();
                if (f0 + 32 <= d) {
#pragma unroll
                    for (int q = 0; q < 32; ++q) acc = __fadd_rn(acc, sq[q][lane]);
                } else {
                    for (int q = 0; q < d - f0; ++q) acc = __fadd_rn(acc, sq[q][lane]);
                }
                __syncwarp();  // sq is overwritten by the next run of features
            }
            if (lane < m) lower(mine, acc);
            __syncwarp();  // frames is overwritten by the next group
        }
    }
    if (!kmpp_last_cta(done)) return;
    if (threadIdx.x == 0) *list_n = 0;  // for the next round
    kmpp_draw_round<kEvalWarps * 32>(ntiles, src, n, d, C0, idx_out, mind, qexp, tile_sum, done, r, seed);
}

// Round 0: a uniformly drawn frame, copied into C0[0].
template <class Src>
__global__ void __launch_bounds__(kTileThreads) kmpp_uniform_kernel(const Src src, int64_t n, int d,
                                                                    float *__restrict__ C0,
                                                                    int64_t *__restrict__ idx_out, uint32_t seed) {
    const int64_t p = (int64_t)__umul64hi(kmpp_draw(seed, 0u), (unsigned long long)n);
    for (int f = threadIdx.x; f < d; f += blockDim.x) C0[f] = src.get(p, f);
    if (idx_out && threadIdx.x == 0) idx_out[0] = p;
}

}  // namespace

size_t kmpp_ws_size(int64_t n, int d, int k) {
    (void)d;
    size_t b = 0;
    carve(nullptr, n, k, &b);
    return b;
}

// The prune factor F for d features: a frame is skipped when
// cc_a >= F mind.  With u = 2^-24, the oracle's sequential float32 distance D
// of a frame to a center lies within (1 -+ u)^(d+3) of the exact squared
// distance (d subtractions, d squares, d additions, each rounded once), and
// the cc kernel's value within (1 +- u)^2 (1 +- g_m) of it, g_m = m u / (1 -
// m u) for its m = ceil(d/32) + 5 roundings per sum.  The exact new distance
// is at least (sqrt(CC) - sqrt(D*))^2 once sqrt(CC) >= sqrt(D*), which gives
// F = 4 (1 + u)^2 (1 + g_m) / (1 - u)^(d+3), enlarged by 2^-20 and rounded up
// to float.
float prune_factor(int d) {
    const double u = std::ldexp(1.0, -24);
    const double mrnd = (double)((d + 31) / 32 + 5);
    const double gm = mrnd * u / (1.0 - mrnd * u);
    const double f = 4.0 * (1.0 + u) * (1.0 + u) * (1.0 + gm) / std::pow(1.0 - u, (double)(d + 3)) *
                     (1.0 + std::ldexp(1.0, -20));
    float ff = (float)f;
    if ((double)ff < f) ff = std::nextafter(ff, 8.0f);
    return ff;
}

namespace {

template <class Src>
int run_kmpp_src(const Src &src, int64_t n, int d, int k, uint32_t seed, float *C0, int64_t *idx,
                 void (*cb)(void *), void *cb_user, void *ws, cudaStream_t s, const KmppMetric &m) {
    KmppWs w = carve(ws, n, k, nullptr);
    const int64_t ntiles = (n + kTile - 1) / kTile;
    kmpp_uniform_kernel<<<1, kTileThreads, 0, s>>>(src, n, d, C0, idx, seed);
    KM_CUDA(cudaGetLastError());
    if (cb) cb(cb_user);
    if (k == 1) return KM_OK;
    KM_CUDA(cudaMemsetAsync(w.maxbits, 0, sizeof(uint32_t), s));
    KM_CUDA(cudaMemsetAsync(w.done, 0, sizeof(unsigned int), s));
    kmpp_first_kernel<<<(unsigned)ntiles, kTileThreads, 0, s>>>(src, n, d, C0, w.mind, w.near, w.maxbits, m);
    KM_CUDA(cudaGetLastError());
    kmpp_scale_kernel<<<1, 1, 0, s>>>(w.maxbits, n, w.qexp);
    KM_CUDA(cudaGetLastError());
    const float pf = prune_factor(d);
    // Pruned rounds pay three launches per round; below this size the
    // unpruned pass is about as short as a launch.  KM_KMPP_PRUNE=0 or 1 in
    // the environment forces the choice (both give the same draws).
    bool prune = !m.Xc && n * (int64_t)d >= (int64_t(1) << 22);
    if (const char *e = std::getenv("KM_KMPP_PRUNE")) prune = !m.Xc && e[0] == '1';
    if (prune) KM_CUDA(cudaMemsetAsync(w.list_n, 0, sizeof(int32_t), s));
    const int64_t nq = (n + 3) / 4;
    const unsigned prune_grid = (unsigned)std::min<int64_t>((nq + 255) / 256, (int64_t)num_sms() * 8);
    const unsigned eval_grid = (unsigned)num_sms() * 4;
    for (int r = 1; r < k; ++r) {
        const int rc = r >= 2 ? r - 1 : -1;
        if (m.Xc) {
            if constexpr (std::is_same<Src, DenseRows>::value)
                kmpp_round_kernel<256, true><<<(unsigned)ntiles, 256, 0, s>>>(src, n, d, C0, idx, w.mind, w.qexp,
                                                                              w.tile_sum, w.done, m, rc, r, seed);
        } else if (!prune || rc < 0) {
            kmpp_round_kernel<1024, false><<<(unsigned)ntiles, 1024, 0, s>>>(src, n, d, C0, idx, w.mind, w.qexp,
                                                                             w.tile_sum, w.done, m, rc, r, seed);
        } else {
            kmpp_cc_kernel<<<(unsigned)((rc + 7) / 8), 256, 0, s>>>(C0, d, rc, w.cc);
            KM_CUDA(cudaGetLastError());
            kmpp_prune_kernel<<<prune_grid, 256, 0, s>>>(n, w.mind, w.near, w.cc, pf, w.list, w.list_n);
            KM_CUDA(cudaGetLastError());
            kmpp_eval_kernel<<<eval_grid, kEvalWarps * 32, 0, s>>>(src, n, d, C0, idx, w.mind, w.near, w.qexp,
                                                                   w.tile_sum, w.done, w.list, w.list_n, ntiles, rc, r,
                                                                   seed);
        }
        KM_CUDA(cudaGetLastError());
        if (cb) cb(cb_user);
    }
    return KM_OK;
}

}  // namespace

int run_kmpp(const float *X, int64_t n, int d, int k, uint32_t seed, float *C0, int64_t *idx,
             void (*cb)(void *), void *cb_user, void *ws, cudaStream_t s, const KmppMetric *metric,
             const PairSrc *ps) {
    const KmppMetric m = metric ? *metric : KmppMetric{nullptr, nullptr, nullptr};
    if (n <= 0) {
        set_error("kmeans++ needs at least one frame");
        return KM_ERR_BAD_SHAPE;
    }
    if (ps) {
        if (m.Xc) {
            set_error("kmeans++ under the minRMSD metric takes dense frames");
            return KM_ERR_UNSUPPORTED;
        }
        const PairRows pr{ps->xyz, reinterpret_cast<const int2 *>(ps->pairs), ps->n_atoms, d};
        return run_kmpp_src(pr, n, d, k, seed, C0, idx, cb, cb_user, ws, s, m);
    }
    return run_kmpp_src(DenseRows{X, d}, n, d, k, seed, C0, idx, cb, cb_user, ws, s, m);
}

}  // namespace km

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
// Pruning (Euclidean metric): each frame keeps, besides D^2 = mind, the index
// a of a center whose exact distance is mind.  Before round r's pass a small
// kernel bounds cc_j = ||c_new - c_j||^2 for every earlier center j.  By the
// triangle inequality ||x - c_new|| >= ||c_new - c_a|| - ||x - c_a||, so when
// cc_a >= 4 mind (times a factor covering the float32 rounding of mind, of
// the new distance and of cc) the exact new distance cannot fall below mind
// and the frame's row is not read.  The running minima, and so the draws,
// are the same as without pruning, bit for bit; a skipped frame costs 8 bytes
// (mind, a) instead of 4d + 4.
#include <climits>
#include <cmath>

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

// Round 1 pass: mind = D^2 to center 0 (near = 0); max of the finite values.
__global__ void __launch_bounds__(kTileThreads) kmpp_first_kernel(
    const float *__restrict__ X, int64_t n, int d, const float *__restrict__ c0,
    float *__restrict__ mind, int32_t *__restrict__ near, uint32_t *__restrict__ maxbits, KmppMetric m) {
    float mx = 0.0f;
    const int64_t t0 = (int64_t)blockIdx.x * kTile;
    for (int u = 0; u < kTile / kTileThreads; ++u) {
        const int64_t i = t0 + u * kTileThreads + threadIdx.x;
        if (i < n) {
            const float dd = kmpp_d2(X, i, d, c0, m, 0);
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

// The end of a round, after the pass: the tile's weight sum s (any thread's
// share) is reduced and stored; the CTA that finishes last draws frame r:
// t = floor(u W / 2^64) for the weight total W, the first frame whose
// inclusive prefix weight exceeds t (a uniform frame when W = 0), copied into
// C0[r].  The other CTAs return.
template <int THREADS>
__device__ __forceinline__ void kmpp_finish_round(unsigned long long s, const float *__restrict__ X, int64_t n,
                                                  int d, float *__restrict__ C0, int64_t *__restrict__ idx_out,
                                                  const float *__restrict__ mind, int qexp,
                                                  unsigned long long *__restrict__ tile_sum,
                                                  unsigned int *__restrict__ done, int r, uint32_t seed) {
    constexpr int kPer = kTile / THREADS;  // frames per thread in the draw's tile
    __shared__ unsigned long long red[THREADS / 32];
    __shared__ bool last;
    __shared__ long long tile_hit, pick;
    __shared__ unsigned long long target;
    s = block_sum_u64(s, red);
    __threadfence();  // this thread's running minimum before the count
    __syncthreads();
    if (threadIdx.x == 0) {
        tile_sum[blockIdx.x] = s;
        __threadfence();
        last = atomicAdd(done, 1u) == gridDim.x - 1;
        tile_hit = -1;
        pick = -1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();

    // The draw (the other CTAs' sums and minima are read past L1).
    const int64_t ntiles = gridDim.x;
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
    for (int f = threadIdx.x; f < d; f += THREADS) C0[(int64_t)r * d + f] = X[p * d + f];
    if (threadIdx.x == 0) {
        if (idx_out) idx_out[r] = p;
        *done = 0u;  // for the next round's launch
    }
}

// The skip test of the pruned pass: the bound shows that the exact distance
// to the new center is at least mi (finite mi only; a NaN bound never skips).
__device__ __forceinline__ bool kmpp_skip(float mi, int32_t a, const float *__restrict__ cc, float prune_factor) {
    return mi <= 3.4028234663852886e38f && __ldg(cc + a) >= __fmul_ru(mi, prune_factor);
}

// Round r >= 1, one CTA per tile of kTile frames, one thread per frame (at
// a time).  With r_center >= 0 the running minimum first takes the distance
// to center r_center (rounds >= 2; round 1 uses the minimum of
// kmpp_first_kernel as it is); PRUNE skips the frames that the bound rules
// out.  Then kmpp_finish_round.  THREADS = 1024 for narrow Euclidean rows
// (two frames per thread: the pass is latency-bound at small n), 256 for
// minRMSD (the QCP solve needs the registers).
template <int THREADS, bool RMSD, bool PRUNE>
__global__ void __launch_bounds__(THREADS) kmpp_round_kernel(
    const float *__restrict__ X, int64_t n, int d, float *__restrict__ C0, int64_t *__restrict__ idx_out,
    float *__restrict__ mind, int32_t *__restrict__ near, const float *__restrict__ cc,
    float prune_factor, const int *__restrict__ qexp_p, unsigned long long *__restrict__ tile_sum,
    unsigned int *__restrict__ done, KmppMetric m, int r_center, int r, uint32_t seed) {
    constexpr int kPer = kTile / THREADS;
    const int qexp = *qexp_p;
    const int64_t t0 = (int64_t)blockIdx.x * kTile;
    unsigned long long s = 0;
    for (int u = 0; u < kPer; ++u) {
        const int64_t i = t0 + u * THREADS + threadIdx.x;
        if (i < n) {
            float mi = mind[i];
            if (r_center >= 0 && !(PRUNE && kmpp_skip(mi, near[i], cc, prune_factor))) {
                const float *c = C0 + (int64_t)r_center * d;
                const float dd = RMSD ? kmpp_d2(X, i, d, c, m, r_center) : sqdist_exact(X + i * d, c, d);
                if (dd < mi) {
                    mi = dd;
                    mind[i] = mi;
                    if (PRUNE) near[i] = r_center;
                }
            }
            s += quant_weight(mi, qexp);
        }
    }
    kmpp_finish_round<THREADS>(s, X, n, d, C0, idx_out, mind, qexp, tile_sum, done, r, seed);
}

// The pruned Euclidean pass for rows of at least 32 features, warp by warp.
// A warp owns 8 windows of 32 frames of the tile; the frames that the bound
// does not rule out are queued in shared memory and evaluated 32 at a time:
// for each 32-feature slice lane l loads feature f0 + l of every queued row
// (coalesced) and of the new center, rounds (x - c)^2 and stores it
// transposed; lane b then adds row b's squares in feature order, which is
// sqdist_exact's sum bit for bit.  One thread per row would make every warp
// load touch 32 rows, and that pass is bound by L1 wavefronts.
constexpr int kWarpThreads = 256;
constexpr int kWarpWin = kTile / kWarpThreads;  // windows of 32 frames per warp

struct KmppWarpSmem {
    float sq[32][33];         // sq[l][b]: rounded square of feature f0 + l of queued row b
    int32_t q[64];            // queued frames (window * 32 + lane)
    float m[kWarpWin * 32];   // the warp's running minima
};

__global__ void __launch_bounds__(kWarpThreads) kmpp_round_warp_kernel(
    const float *__restrict__ X, int64_t n, int d, float *__restrict__ C0, int64_t *__restrict__ idx_out,
    float *__restrict__ mind, int32_t *__restrict__ near, const float *__restrict__ cc, float prune_factor,
    const int *__restrict__ qexp_p, unsigned long long *__restrict__ tile_sum, unsigned int *__restrict__ done,
    int r_center, int r, uint32_t seed) {
    __shared__ KmppWarpSmem wsm[kWarpThreads / 32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    KmppWarpSmem &w = wsm[warp];
    const int qexp = *qexp_p;
    const int64_t t0 = (int64_t)blockIdx.x * kTile + warp * 32;  // frame of window 0, lane 0
    const float *c = C0 + (int64_t)(r_center > 0 ? r_center : 0) * d;

    auto process = [&](int nb) {
        float acc = 0.0f;
        for (int f0 = 0; f0 < d; f0 += 32) {
            const int f = f0 + lane;
            if (f < d) {
                const float cf = __ldg(c + f);
#pragma unroll 8
                for (int b = 0; b < 32; ++b) {
                    if (b < nb) {
                        const int li = w.q[b];
                        const int64_t i = t0 + (int64_t)(li >> 5) * kWarpThreads + (li & 31);
                        w.sq[lane][b] = sq_term(__ldg(X + i * d + f), cf);
                    }
                }
            }
            __syncwarp();
            const int fw = min(32, d - f0);
            if (lane < nb)
                for (int l = 0; l < fw; ++l) acc = __fadd_rn(acc, w.sq[l][lane]);
            __syncwarp();
        }
        if (lane < nb) {
            const int li = w.q[lane];
            if (acc < w.m[li]) {
                const int64_t i = t0 + (int64_t)(li >> 5) * kWarpThreads + (li & 31);
                w.m[li] = acc;
                mind[i] = acc;
                near[i] = r_center;
            }
        }
        __syncwarp();
    };

    int qn = 0;  // queued frames (warp-uniform)
    for (int u = 0; u < kWarpWin; ++u) {
        const int64_t i = t0 + (int64_t)u * kWarpThreads + lane;
        const int li = u * 32 + lane;
        bool act = false;
        float mi = 0.0f;
        if (i < n) {
            mi = mind[i];
            act = r_center >= 0 && !kmpp_skip(mi, near[i], cc, prune_factor);
        }
        w.m[li] = mi;
        const unsigned msk = __ballot_sync(0xffffffffu, act);
        if (act) w.q[qn + __popc(msk & ((1u << lane) - 1u))] = li;
        qn += __popc(msk);
        __syncwarp();
        if (qn >= 32) {
            process(32);
            qn -= 32;
            if (lane < qn) w.q[lane] = w.q[32 + lane];  // slots 32 .. 32 + qn move to the front
            __syncwarp();
        }
    }
    if (qn > 0) process(qn);
    unsigned long long s = 0;
    for (int u = 0; u < kWarpWin; ++u)
        if (t0 + (int64_t)u * kWarpThreads + lane < n) s += quant_weight(w.m[u * 32 + lane], qexp);
    kmpp_finish_round<kWarpThreads>(s, X, n, d, C0, idx_out, mind, qexp, tile_sum, done, r, seed);
}

// Round 0: a uniformly drawn frame, copied into C0[0].
__global__ void __launch_bounds__(kTileThreads) kmpp_uniform_kernel(const float *__restrict__ X, int64_t n, int d,
                                                                    float *__restrict__ C0,
                                                                    int64_t *__restrict__ idx_out, uint32_t seed) {
    const int64_t p = (int64_t)__umul64hi(kmpp_draw(seed, 0u), (unsigned long long)n);
    for (int f = threadIdx.x; f < d; f += blockDim.x) C0[f] = X[p * d + f];
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

int run_kmpp(const float *X, int64_t n, int d, int k, uint32_t seed, float *C0, int64_t *idx,
             void (*cb)(void *), void *cb_user, void *ws, cudaStream_t s, const KmppMetric *metric) {
    const KmppMetric m = metric ? *metric : KmppMetric{nullptr, nullptr, nullptr};
    if (n <= 0) {
        set_error("kmeans++ needs at least one frame");
        return KM_ERR_BAD_SHAPE;
    }
    KmppWs w = carve(ws, n, k, nullptr);
    const int64_t ntiles = (n + kTile - 1) / kTile;
    kmpp_uniform_kernel<<<1, kTileThreads, 0, s>>>(X, n, d, C0, idx, seed);
    KM_CUDA(cudaGetLastError());
    if (cb) cb(cb_user);
    if (k == 1) return KM_OK;
    KM_CUDA(cudaMemsetAsync(w.maxbits, 0, sizeof(uint32_t), s));
    KM_CUDA(cudaMemsetAsync(w.done, 0, sizeof(unsigned int), s));
    kmpp_first_kernel<<<(unsigned)ntiles, kTileThreads, 0, s>>>(X, n, d, C0, w.mind, w.near, w.maxbits, m);
    KM_CUDA(cudaGetLastError());
    kmpp_scale_kernel<<<1, 1, 0, s>>>(w.maxbits, n, w.qexp);
    KM_CUDA(cudaGetLastError());
    const float pf = prune_factor(d);
    for (int r = 1; r < k; ++r) {
        const int rc = r >= 2 ? r - 1 : -1;
        if (m.Xc) {
            kmpp_round_kernel<256, true, false><<<(unsigned)ntiles, 256, 0, s>>>(
                X, n, d, C0, idx, w.mind, w.near, w.cc, pf, w.qexp, w.tile_sum, w.done, m, rc, r, seed);
        } else {
            if (rc >= 1) {
                kmpp_cc_kernel<<<(unsigned)((rc + 7) / 8), 256, 0, s>>>(C0, d, rc, w.cc);
                KM_CUDA(cudaGetLastError());
            }
            if (d >= 32)
                kmpp_round_warp_kernel<<<(unsigned)ntiles, kWarpThreads, 0, s>>>(
                    X, n, d, C0, idx, w.mind, w.near, w.cc, pf, w.qexp, w.tile_sum, w.done, rc, r, seed);
            else
                kmpp_round_kernel<1024, false, true><<<(unsigned)ntiles, 1024, 0, s>>>(
                    X, n, d, C0, idx, w.mind, w.near, w.cc, pf, w.qexp, w.tile_sum, w.done, m, rc, r, seed);
        }
        KM_CUDA(cudaGetLastError());
        if (cb) cb(cb_user);
    }
    return KM_OK;
}

}  // namespace km

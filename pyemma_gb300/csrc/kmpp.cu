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
#include "km_common.cuh"
#include "km_internal.h"
#include "km_rmsd.cuh"

namespace km {

namespace {

constexpr int kTile = 2048;  // frames per weight tile
constexpr int kTileThreads = 256;

struct KmppWs {
    float *mind;
    unsigned long long *tile_sum;
    uint32_t *maxbits;
    double *scale;
    unsigned int *done;  // CTAs of the current round that have finished
};

KmppWs carve(void *ws, int64_t n, size_t *bytes) {
    Carver c(ws);
    KmppWs w;
    const int64_t ntiles = (n + kTile - 1) / kTile;
    w.mind = c.take<float>(n > 0 ? n : 1);
    w.tile_sum = c.take<unsigned long long>(ntiles > 0 ? ntiles : 1);
    w.maxbits = c.take<uint32_t>(1);
    w.scale = c.take<double>(1);
    w.done = c.take<unsigned int>(1);
    if (bytes) *bytes = c.bytes();
    return w;
}

__device__ __forceinline__ unsigned long long quant_weight(float w, double scale) {
    if (!(w > 0.0f) || w == __int_as_float(0x7f800000)) return 0ull;
    return (unsigned long long)((double)w * scale);
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

// Round 1 pass: mind = D^2 to center 0; max of the finite values.
__global__ void __launch_bounds__(kTileThreads) kmpp_first_kernel(
    const float *__restrict__ X, int64_t n, int d, const float *__restrict__ c0,
    float *__restrict__ mind, uint32_t *__restrict__ maxbits, KmppMetric m) {
    float mx = 0.0f;
    const int64_t t0 = (int64_t)blockIdx.x * kTile;
    for (int u = 0; u < kTile / kTileThreads; ++u) {
        const int64_t i = t0 + u * kTileThreads + threadIdx.x;
        if (i < n) {
            const float dd = kmpp_d2(X, i, d, c0, m, 0);
            mind[i] = dd;
            if (dd < __int_as_float(0x7f800000) && dd > mx) mx = dd;
        }
    }
    for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    if ((threadIdx.x & 31) == 0 && mx > 0.0f) atomicMax(maxbits, __float_as_uint(mx));
}

// e = 62 - ceil(log2 n) - E(max) with 2^(E-1) <= max < 2^E; scale = 2^e.
__global__ void kmpp_scale_kernel(const uint32_t *__restrict__ maxbits, int64_t n,
                                  double *__restrict__ scale) {
    const uint32_t b = *maxbits;
    const float m = __uint_as_float(b);
    if (!(m > 0.0f) || m == __int_as_float(0x7f800000)) {
        *scale = 0.0;
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
    const int e = 62 - L - E;
    *scale = __longlong_as_double((long long)(e + 1023) << 52);
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

// Round r >= 1, one CTA per tile of kTile frames.  With r_center >= 0 the
// running minimum first takes the distance to center r_center (rounds >= 2;
// round 1 uses the minimum of kmpp_first_kernel as it is).  Then the tile's
// weight sum; the CTA that finishes last draws frame r: t = floor(u W / 2^64)
// for the weight total W, the first frame whose inclusive prefix weight
// exceeds t (a uniform frame when W = 0), copied into C0[r].  THREADS = 1024
// for the Euclidean metric (two frames per thread: the pass is latency-bound
// at small n), 256 for minRMSD (the QCP solve needs the registers).
template <int THREADS, bool RMSD>
__global__ void __launch_bounds__(THREADS) kmpp_round_kernel(
    const float *__restrict__ X, int64_t n, int d, float *__restrict__ C0, int64_t *__restrict__ idx_out,
    float *__restrict__ mind, const double *__restrict__ scale_p, unsigned long long *__restrict__ tile_sum,
    unsigned int *__restrict__ done, KmppMetric m, int r_center, int r, uint32_t seed) {
    constexpr int kPer = kTile / THREADS;  // frames per thread in the pass and in the draw's tile
    __shared__ unsigned long long red[THREADS / 32];
    __shared__ bool last;
    __shared__ long long tile_hit, pick;
    __shared__ unsigned long long target;
    const double scale = *scale_p;
    const int64_t t0 = (int64_t)blockIdx.x * kTile;
    unsigned long long s = 0;
    for (int u = 0; u < kPer; ++u) {
        const int64_t i = t0 + u * THREADS + threadIdx.x;
        if (i < n) {
            float mi = mind[i];
            if (r_center >= 0) {
                const float *c = C0 + (int64_t)r_center * d;
                const float dd = RMSD ? kmpp_d2(X, i, d, c, m, r_center) : sqdist_exact(X + i * d, c, d);
                if (dd < mi) {
                    mi = dd;
                    mind[i] = mi;
                }
            }
            s += quant_weight(mi, scale);
        }
    }
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
            w[q] = f0 + q < n ? quant_weight(__ldcg(mind + f0 + q), scale) : 0ull;
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
    (void)k;
    size_t b = 0;
    carve(nullptr, n, &b);
    return b;
}

int run_kmpp(const float *X, int64_t n, int d, int k, uint32_t seed, float *C0, int64_t *idx,
             void (*cb)(void *), void *cb_user, void *ws, cudaStream_t s, const KmppMetric *metric) {
    const KmppMetric m = metric ? *metric : KmppMetric{nullptr, nullptr, nullptr};
    if (n <= 0) {
        set_error("kmeans++ needs at least one frame");
        return KM_ERR_BAD_SHAPE;
    }
    KmppWs w = carve(ws, n, nullptr);
    const int64_t ntiles = (n + kTile - 1) / kTile;
    kmpp_uniform_kernel<<<1, kTileThreads, 0, s>>>(X, n, d, C0, idx, seed);
    KM_CUDA(cudaGetLastError());
    if (cb) cb(cb_user);
    if (k == 1) return KM_OK;
    KM_CUDA(cudaMemsetAsync(w.maxbits, 0, sizeof(uint32_t), s));
    KM_CUDA(cudaMemsetAsync(w.done, 0, sizeof(unsigned int), s));
    kmpp_first_kernel<<<(unsigned)ntiles, kTileThreads, 0, s>>>(X, n, d, C0, w.mind, w.maxbits, m);
    KM_CUDA(cudaGetLastError());
    kmpp_scale_kernel<<<1, 1, 0, s>>>(w.maxbits, n, w.scale);
    KM_CUDA(cudaGetLastError());
    for (int r = 1; r < k; ++r) {
        const int rc = r >= 2 ? r - 1 : -1;
        if (m.Xc)
            kmpp_round_kernel<256, true><<<(unsigned)ntiles, 256, 0, s>>>(X, n, d, C0, idx, w.mind, w.scale,
                                                                          w.tile_sum, w.done, m, rc, r, seed);
        else
            kmpp_round_kernel<1024, false><<<(unsigned)ntiles, 1024, 0, s>>>(X, n, d, C0, idx, w.mind, w.scale,
                                                                             w.tile_sum, w.done, m, rc, r, seed);
        KM_CUDA(cudaGetLastError());
        if (cb) cb(cb_user);
    }
    return KM_OK;
}

}  // namespace km

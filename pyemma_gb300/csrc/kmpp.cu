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
// Per round: one pass over X (distance to the newest center, running minimum,
// per-tile weight sums; HBM-bound) and one single-CTA pick kernel.
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
};

KmppWs carve(void *ws, int64_t n, size_t *bytes) {
    Carver c(ws);
    KmppWs w;
    const int64_t ntiles = (n + kTile - 1) / kTile;
    w.mind = c.take<float>(n > 0 ? n : 1);
    w.tile_sum = c.take<unsigned long long>(ntiles > 0 ? ntiles : 1);
    w.maxbits = c.take<uint32_t>(1);
    w.scale = c.take<double>(1);
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

// Weight tile sums from mind (round 1).
__global__ void __launch_bounds__(kTileThreads) kmpp_weights_kernel(
    const float *__restrict__ mind, int64_t n, const double *__restrict__ scale_p,
    unsigned long long *__restrict__ tile_sum) {
    __shared__ unsigned long long red[kTileThreads / 32];
    const double scale = *scale_p;
    const int64_t t0 = (int64_t)blockIdx.x * kTile;
    unsigned long long s = 0;
    for (int u = 0; u < kTile / kTileThreads; ++u) {
        const int64_t i = t0 + u * kTileThreads + threadIdx.x;
        if (i < n) s += quant_weight(mind[i], scale);
    }
    s = block_sum_u64(s, red);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = s;
}

// Rounds >= 2: update the running minimum with the newest center, then
// weight tile sums.
__global__ void __launch_bounds__(kTileThreads) kmpp_round_kernel(
    const float *__restrict__ X, int64_t n, int d, const float *__restrict__ c,
    float *__restrict__ mind, const double *__restrict__ scale_p,
    unsigned long long *__restrict__ tile_sum, KmppMetric m, int r_center) {
    __shared__ unsigned long long red[kTileThreads / 32];
    const double scale = *scale_p;
    const int64_t t0 = (int64_t)blockIdx.x * kTile;
    unsigned long long s = 0;
    for (int u = 0; u < kTile / kTileThreads; ++u) {
        const int64_t i = t0 + u * kTileThreads + threadIdx.x;
        if (i < n) {
            const float dd = kmpp_d2(X, i, d, c, m, r_center);
            float mi = mind[i];
            if (dd < mi) {
                mi = dd;
                mind[i] = mi;
            }
            s += quant_weight(mi, scale);
        }
    }
    s = block_sum_u64(s, red);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = s;
}

// Single CTA of 1024 threads: draw round r and copy the chosen frame into
// C0[r].  uniform != 0 draws a frame uniformly (round 0).
__global__ void __launch_bounds__(1024) kmpp_pick_kernel(
    const float *__restrict__ X, int64_t n, int d, float *__restrict__ C0,
    int64_t *__restrict__ idx_out, int r, uint32_t seed, int uniform,
    const float *__restrict__ mind, const double *__restrict__ scale_p,
    const unsigned long long *__restrict__ tile_sum, int64_t ntiles) {
    __shared__ unsigned long long part[1024];
    __shared__ long long pick;
    __shared__ unsigned long long target;
    __shared__ long long tile_hit;
    const int tid = threadIdx.x;
    const uint64_t u = kmpp_draw(seed, (uint32_t)r);
    if (tid == 0) {
        pick = -1;
        tile_hit = -1;
    }
    if (!uniform) {
        // Total weight and the tile holding the target.
        const int64_t per = (ntiles + 1023) / 1024;
        const int64_t lo = tid * per, hi = min(lo + per, ntiles);
        unsigned long long s = 0;
        for (int64_t b = lo; b < hi; ++b) s += tile_sum[b];
        part[tid] = s;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            unsigned long long v = tid >= off ? part[tid - off] : 0ull;
            __syncthreads();
            part[tid] += v;
            __syncthreads();
        }
        const unsigned long long total = part[1023];
        if (total > 0) {
            const unsigned long long t = __umul64hi(u, total);
            unsigned long long run = part[tid] - s;  // exclusive prefix of this thread's range
            if (run <= t && t < part[tid]) {
                for (int64_t b = lo; b < hi; ++b) {
                    if (t < run + tile_sum[b]) {
                        tile_hit = b;
                        target = t - run;
                        break;
                    }
                    run += tile_sum[b];
                }
            }
        }
        __syncthreads();
        if (tile_hit >= 0) {
            // Inside the tile: two frames per thread, inclusive scan.
            const double scale = *scale_p;
            const int64_t f0 = tile_hit * kTile + 2 * tid;
            const unsigned long long w0 = f0 < n ? quant_weight(mind[f0], scale) : 0ull;
            const unsigned long long w1 = f0 + 1 < n ? quant_weight(mind[f0 + 1], scale) : 0ull;
            __syncthreads();
            part[tid] = w0 + w1;
            __syncthreads();
            for (int off = 1; off < 1024; off <<= 1) {
                unsigned long long v = tid >= off ? part[tid - off] : 0ull;
                __syncthreads();
                part[tid] += v;
                __syncthreads();
            }
            const unsigned long long incl = part[tid];
            const unsigned long long excl = incl - w0 - w1;
            const unsigned long long tt = target;
            if (excl <= tt && tt < incl) pick = (tt < excl + w0) ? f0 : f0 + 1;
        }
    }
    __syncthreads();
    if (pick < 0 && tid == 0) pick = (long long)__umul64hi(u, (unsigned long long)n);
    __syncthreads();
    const int64_t p = pick;
    for (int f = tid; f < d; f += 1024) C0[(int64_t)r * d + f] = X[p * d + f];
    if (idx_out && tid == 0) idx_out[r] = p;
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
    kmpp_pick_kernel<<<1, 1024, 0, s>>>(X, n, d, C0, idx, 0, seed, 1, w.mind, w.scale, w.tile_sum,
                                        ntiles);
    KM_CUDA(cudaGetLastError());
    if (cb) cb(cb_user);
    if (k == 1) return KM_OK;
    KM_CUDA(cudaMemsetAsync(w.maxbits, 0, sizeof(uint32_t), s));
    kmpp_first_kernel<<<(unsigned)ntiles, kTileThreads, 0, s>>>(X, n, d, C0, w.mind, w.maxbits, m);
    KM_CUDA(cudaGetLastError());
    kmpp_scale_kernel<<<1, 1, 0, s>>>(w.maxbits, n, w.scale);
    KM_CUDA(cudaGetLastError());
    kmpp_weights_kernel<<<(unsigned)ntiles, kTileThreads, 0, s>>>(w.mind, n, w.scale, w.tile_sum);
    KM_CUDA(cudaGetLastError());
    for (int r = 1; r < k; ++r) {
        if (r >= 2) {
            kmpp_round_kernel<<<(unsigned)ntiles, kTileThreads, 0, s>>>(
                X, n, d, C0 + (int64_t)(r - 1) * d, w.mind, w.scale, w.tile_sum, m, r - 1);
            KM_CUDA(cudaGetLastError());
        }
        kmpp_pick_kernel<<<1, 1024, 0, s>>>(X, n, d, C0, idx, r, seed, 0, w.mind, w.scale, w.tile_sum,
                                            ntiles);
        KM_CUDA(cudaGetLastError());
        if (cb) cb(cb_user);
    }
    return KM_OK;
}

}  // namespace km

// update.cu -- kernel (c): centroid update and inertia in float64.
//
// Reference: the M-step of KMeans.fit, pyemma/coordinates/clustering/
// kmeans.py:253-258 (new center = mean of its members; the cost function of
// kmeans.py:71-75 evaluated for the new centers).  An empty cluster keeps its
// previous center.
//
// Frames are grouped by label with a counting sort (histogram, exclusive
// scan, warp-aggregated scatter of frame indices and their labels).  Warps
// then walk the sorted list in pieces of 256 positions; inside a piece
// consecutive frames mostly share a label, so per-lane compensated float32
// sums accumulate a run and flush it into the float64 totals with one atomic
// add per feature when the label changes.  The number of global atomics is
// about (pieces + k) * d instead of n * d, and no per-element float64
// arithmetic is needed.  Each deviation x - c_j is rounded once to float32.
//
// Sums are taken relative to the previous center c_j of each cluster:
//   S_j = sum (x_i - c_j),  Q_j = sum ||x_i - c_j||^2,
//   mu_j = float(c_j + S_j / n_j),  delta_j = mu_j - c_j,
//   inertia_j = Q_j - 2 delta_j . S_j + n_j ||delta_j||^2
// which is sum_i ||x_i - mu_j||^2 without the cancellation of raw moments.
#include <algorithm>
#include <map>
#include <mutex>

#include "km_common.cuh"
#include "km_internal.h"

namespace km {

namespace {

constexpr int kPiece = 256;     // sorted positions per warp (8 groups of 32)
constexpr int kGroups = kPiece / 32;

struct UpdateWs {
    int32_t *counts;
    int32_t *total;  // members over several parts (launch_update_part)
    int32_t *offsets;
    int32_t *cursor;
    int32_t *perm;
    int32_t *slab;
    double *S;
    double *Q;
    double *ccost;
};

UpdateWs carve(void *ws, int64_t n, int d, int k, size_t *bytes) {
    Carver c(ws);
    UpdateWs u;
    u.counts = c.take<int32_t>(k);
    u.total = c.take<int32_t>(k);
    u.offsets = c.take<int32_t>((size_t)k + 1);
    u.cursor = c.take<int32_t>(k);
    u.perm = c.take<int32_t>(n > 0 ? n : 1);
    u.slab = c.take<int32_t>(n > 0 ? n : 1);
    u.S = c.take<double>((size_t)k * d);
    u.Q = c.take<double>(k);
    u.ccost = c.take<double>(k);
    if (bytes) *bytes = c.bytes();
    return u;
}

__global__ void count_labels_kernel(const int32_t *__restrict__ labels, int64_t n, int k,
                                    int32_t *__restrict__ counts, uint32_t *err) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        int l = i < n ? labels[i] : -1;
        if (i < n && (l < 0 || l >= k)) {
            atomicOr(err, (uint32_t)kDevBadLabel);
            l = -1;
        }
        const unsigned peers = __match_any_sync(0xffffffffu, l);
        if (l >= 0 && lane == __ffs(peers) - 1) atomicAdd(&counts[l], __popc(peers));
    }
}

// Single CTA: exclusive scan of counts into offsets[0..k] and cursor.
__global__ void __launch_bounds__(1024) scan_counts_kernel(const int32_t *__restrict__ counts, int k,
                                                            int32_t *__restrict__ offsets,
                                                            int32_t *__restrict__ cursor) {
    __shared__ int32_t part[1024];
    const int per = (k + blockDim.x - 1) / blockDim.x;
    const int lo = threadIdx.x * per;
    const int hi = min(lo + per, k);
    int32_t s = 0;
    for (int j = lo; j < hi; ++j) s += counts[j];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < (int)blockDim.x; off <<= 1) {
        int32_t v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    int32_t run = part[threadIdx.x] - s;
    for (int j = lo; j < hi; ++j) {
        offsets[j] = run;
        cursor[j] = run;
        run += counts[j];
    }
    if (threadIdx.x == blockDim.x - 1) offsets[k] = part[threadIdx.x];
}

__global__ void scatter_kernel(const int32_t *__restrict__ labels, int64_t n, int k,
                               int32_t *__restrict__ cursor, int32_t *__restrict__ perm,
                               int32_t *__restrict__ slab) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        int l = i < n ? labels[i] : -1;
        if (l >= k) l = -1;
        const unsigned peers = __match_any_sync(0xffffffffu, l);
        const int leader = __ffs(peers) - 1;
        int pos = 0;
        if (l >= 0 && lane == leader) pos = atomicAdd(&cursor[l], __popc(peers));
        pos = __shfl_sync(0xffffffffu, pos, leader);
        if (l >= 0) {
            const int at = pos + __popc(peers & ((1u << lane) - 1u));
            perm[at] = (int32_t)i;
            slab[at] = l;
        }
    }
}

// The whole warp walks one sorted row at a time; lane covers features
// f_base + lane + 32 m (m < MW); frames wider than 1024 features take one
// launch per 1024-feature slice.  Indices and labels of the piece
// sit in registers (8 per lane) and are broadcast by shuffles; label changes
// are warp-uniform.
template <int MW, class Src>
__global__ void __launch_bounds__(256) seg_accumulate_wide_kernel(
    const Src src, int d, int f_base, const int32_t *__restrict__ perm,
    const int32_t *__restrict__ slab, int64_t n_max, const int32_t *__restrict__ n_sorted,
    const float *__restrict__ C_old, double *__restrict__ S, double *__restrict__ Q) {
    // Only the frames the scatter placed (valid labels) are in perm.
    const int64_t n = min(n_max, (int64_t)*n_sorted);
    const int lane = threadIdx.x & 31;
    const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t npieces = (n + kPiece - 1) / kPiece;
    for (int64_t piece = gwarp; piece < npieces; piece += nwarps) {
        const int64_t p0 = piece * kPiece;
        int my_i[kGroups], my_l[kGroups];
#pragma unroll
        for (int g = 0; g < kGroups; ++g) {
            const int64_t p = p0 + 32 * g + lane;
            my_i[g] = p < n ? perm[p] : 0;
            my_l[g] = p < n ? slab[p] : -1;
        }
        CSum acc[MW], qacc;
        float cold[MW];
        int cur = -1;
        auto flush = [&]() {
#pragma unroll
            for (int m = 0; m < MW; ++m) {
                const int f = f_base + lane + 32 * m;
                if (f < d) atomicAdd(&S[(int64_t)cur * d + f], acc[m].value());
            }
            double q = qacc.value();
            for (int off = 16; off > 0; off >>= 1) q += __shfl_xor_sync(0xffffffffu, q, off);
            if (lane == 0) atomicAdd(&Q[cur], q);
        };
#pragma unroll
        for (int g = 0; g < kGroups; ++g) {
            for (int r = 0; r < 32; ++r) {
                const int l = __shfl_sync(0xffffffffu, my_l[g], r);
                if (l < 0) break;
                const int64_t i = __shfl_sync(0xffffffffu, my_i[g], r);
                if (l != cur) {
                    if (cur >= 0) flush();
                    cur = l;
                    qacc.reset();
#pragma unroll
                    for (int m = 0; m < MW; ++m) {
                        const int f = f_base + lane + 32 * m;
                        acc[m].reset();
                        cold[m] = f < d ? __ldg(C_old + (int64_t)l * d + f) : 0.0f;
                    }
                }
                float xv[MW];
#pragma unroll
                for (int m = 0; m < MW; ++m) {
                    const int f = f_base + lane + 32 * m;
                    xv[m] = f < d ? src.get(i, f) : 0.0f;
                }
#pragma unroll
                for (int m = 0; m < MW; ++m) {
                    const int f = f_base + lane + 32 * m;
                    if (f < d) {
                        const float t = xv[m] - cold[m];
                        acc[m].add(t);
                        qacc.add(t * t);
                    }
                }
            }
        }
        if (cur >= 0) flush();
    }
}

// ---------------------------------------------------------------------------
// Row gathers through 1-D bulk copies (TMA).  The random row reads of the
// sorted walk are latency bound: a warp that loads a row into registers has
// one row in flight.  Here each warp keeps kRing rows in flight in a ring of
// shared-memory row buffers filled by cp.async.bulk (no registers held), and
// reads the features from shared memory.  Needs rows of 16-byte multiples
// (d % 4 == 0) and a 16-byte aligned X.
// ---------------------------------------------------------------------------
constexpr int kRing = 4;
constexpr int kBulkWarps = 8;

__device__ __forceinline__ uint32_t sh_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ring_bar_init(uint64_t *b) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sh_addr(b)) : "memory");
}

__device__ __forceinline__ bool ring_bar_try(uint64_t *b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(sh_addr(b)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait (kWaitLimitNs); false when it gave up.
__device__ __forceinline__ bool ring_bar_wait(uint64_t *b, uint32_t parity) {
    if (ring_bar_try(b, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t spin = 1;; ++spin) {
        if (ring_bar_try(b, parity)) return true;
        if ((spin & 255u) == 0 && globaltimer_ns() - t0 > kWaitLimitNs) return false;
    }
}

// One row into a ring slot; the slot's barrier completes when it has landed.
__device__ __forceinline__ void ring_fetch(void *dst, const void *src, uint32_t bytes, uint64_t *b) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sh_addr(b)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     sh_addr(dst)),
                 "l"(src), "r"(bytes), "r"(sh_addr(b))
                 : "memory");
}

// Ring rows hold MW*32 floats (zero beyond d), so the inner loop needs no
// bounds test.
size_t bulk_smem_bytes(int mw, int ring) {
    return (size_t)kBulkWarps * ((size_t)ring * mw * 128 + 2 * kPiece * 4 + ring * 8);
}

template <int MW, int RING>
__global__ void __launch_bounds__(kBulkWarps * 32, (MW > 17 ? 1 : 2)) seg_accumulate_bulk_kernel(
    const float *__restrict__ X, int d, const int32_t *__restrict__ perm, const int32_t *__restrict__ slab,
    int64_t n_max, const int32_t *__restrict__ n_sorted, const float *__restrict__ C_old, double *__restrict__ S,
    double *__restrict__ Q, uint32_t *err) {
    extern __shared__ __align__(16) unsigned char smem_bulk[];
    constexpr int RS = MW * 32;  // ring row stride (floats)
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t row_bytes = (uint32_t)d * 4u;
    unsigned char *wbase = smem_bulk + (size_t)warp * ((size_t)RING * RS * 4 + 2 * kPiece * 4 + RING * 8);
    float *ring = reinterpret_cast<float *>(wbase);
    int32_t *pidx = reinterpret_cast<int32_t *>(wbase + (size_t)RING * RS * 4);
    int32_t *plab = pidx + kPiece;
    uint64_t *bars = reinterpret_cast<uint64_t *>(plab + kPiece);
    for (int e = lane; e < RING * RS; e += 32) ring[e] = 0.0f;  // the tails beyond d stay zero
    if (lane == 0) {
        for (int r = 0; r < RING; ++r) ring_bar_init(&bars[r]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    uint32_t phase = 0;  // bit r: parity of the next completion of bars[r]
    bool ok = true;

    const int64_t n = min(n_max, (int64_t)*n_sorted);
    const int64_t gwarp = (int64_t)blockIdx.x * kBulkWarps + warp;
    const int64_t nwarps = (int64_t)gridDim.x * kBulkWarps;
    const int64_t npieces = (n + kPiece - 1) / kPiece;
    for (int64_t piece = gwarp; piece < npieces && ok; piece += nwarps) {
        const int64_t p0 = piece * kPiece;
        const int cnt = (int)min((int64_t)kPiece, n - p0);
        for (int q = lane; q < cnt; q += 32) {
            pidx[q] = perm[p0 + q];
            plab[q] = slab[p0 + q];
        }
        __syncwarp();
        int issued = 0;
        auto issue = [&](int q) {  // the whole warp calls; lane 0 issues
            if (lane == 0) {
                const int slot = q & (RING - 1);
                ring_fetch(ring + (size_t)slot * RS, X + (int64_t)pidx[q] * d, row_bytes, &bars[slot]);
            }
            ++issued;
        };
        for (int q = 0; q < cnt && q < RING; ++q) issue(q);

        // Per feature a Kahan sum (ks, kc: the sum is ks - kc); per row the
        // squared deviations of the lane's features in two FMA chains, added
        // to a compensated row total.
        float ks[MW], kc[MW], cold[MW];
        CSum qacc;
        int cur = -1;
        auto flush = [&]() {
#pragma unroll
            for (int m = 0; m < MW; ++m) {
                const int f = lane + 32 * m;
                if (f < d) atomicAdd(&S[(int64_t)cur * d + f], (double)ks[m] - (double)kc[m]);
            }
            double qq = qacc.value();
            for (int off = 16; off > 0; off >>= 1) qq += __shfl_xor_sync(0xffffffffu, qq, off);
            if (lane == 0) atomicAdd(&Q[cur], qq);
        };
        int q = 0;
        for (; q < cnt; ++q) {
            const int slot = q & (RING - 1);
            ok = __all_sync(0xffffffffu, ring_bar_wait(&bars[slot], (phase >> slot) & 1u));
            if (!ok) break;
            phase ^= 1u << slot;
            const int l = plab[q];
            if (l != cur) {
                if (cur >= 0) flush();
                cur = l;
                qacc.reset();
#pragma unroll
                for (int m = 0; m < MW; ++m) {
                    const int f = lane + 32 * m;
                    ks[m] = 0.0f;
                    kc[m] = 0.0f;
                    cold[m] = f < d ? __ldg(C_old + (int64_t)l * d + f) : 0.0f;
                }
            }
            const float *row = ring + (size_t)slot * RS;
            float q0 = 0.0f, q1 = 0.0f;
#pragma unroll
            for (int m = 0; m < MW; ++m) {
                const float t = __fsub_rn(row[lane + 32 * m], cold[m]);  // zero beyond d
                const float y = __fsub_rn(t, kc[m]);
                const float sn = __fadd_rn(ks[m], y);
                kc[m] = __fsub_rn(__fsub_rn(sn, ks[m]), y);
                ks[m] = sn;
                if (m & 1)
                    q1 = __fmaf_rn(t, t, q1);
                else
                    q0 = __fmaf_rn(t, t, q0);
            }
            qacc.add(q0 + q1);
            __syncwarp();
            if (q + RING < cnt) {
                // The slot's shared-memory reads above come before the copy
                // that overwrites it.
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(q + RING);
            }
        }
        if (cur >= 0 && ok) flush();
        if (!ok) {
            // Let the copies still in flight land before the CTA exits.
            for (int r = q; r < issued; ++r) {
                const int slot = r & (RING - 1);
                ring_bar_wait(&bars[slot], (phase >> slot) & 1u);
                phase ^= 1u << slot;
            }
            if (lane == 0) atomicOr(err, (uint32_t)kDevTimeoutTma);
        }
        __syncwarp();
    }
}

// d < 32: the warp is split into 32/DP row slots of DP lanes (DP = next
// power of two >= d); slot s walks positions p0+s, p0+s+R, ...
// ---------------------------------------------------------------------------
// Segment sums of coordinate frames (pair features).  The walk of
// seg_accumulate_wide_kernel, with the coordinates of each sorted frame
// staged in a ring of kPairSlots per-warp shared-memory slots by 4-byte
// cp.async copies, kPairSlots - 1 frames ahead (a frame's 12 n_atoms bytes
// are not a 16-byte multiple, so no bulk copy), and each lane's atom pairs
// held in registers as offsets into a slot (two 16-bit halves).  The
// features are those of PairRows (pair_feature).
// ---------------------------------------------------------------------------
constexpr int kPairSlots = 4;
constexpr int kPairMaxAtoms = 128;  // slots of up to 384 floats: 48 KB per CTA at most

int pair_slot_floats(int n_atoms) { return (3 * n_atoms + 3) & ~3; }
size_t pair_seg_smem(int n_atoms) { return (size_t)8 * kPairSlots * pair_slot_floats(n_atoms) * sizeof(float); }

template <int MW>
__global__ void __launch_bounds__(256) seg_accumulate_pairs_kernel(
    const PairRows src, int d, int f_base, const int32_t *__restrict__ perm, const int32_t *__restrict__ slab,
    int64_t n_max, const int32_t *__restrict__ n_sorted, const float *__restrict__ C_old, double *__restrict__ S,
    double *__restrict__ Q) {
    extern __shared__ float pair_ring[];
    const int64_t n = min(n_max, (int64_t)*n_sorted);
    const int lane = threadIdx.x & 31;
    const int row_floats = 3 * src.n_atoms;
    const int slot = (row_floats + 3) & ~3;
    float *ring = pair_ring + (threadIdx.x >> 5) * kPairSlots * slot;
    const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t npieces = (n + kPiece - 1) / kPiece;
    uint32_t ofs[MW];  // 3 a | 3 b << 16 of the lane's pair m
#pragma unroll
    for (int m = 0; m < MW; ++m) {
        const int f = f_base + lane + 32 * m;
        ofs[m] = 0u;
        if (f < d) {
            const int2 pr = __ldg(src.pairs + f);
            ofs[m] = (uint32_t)(3 * pr.x) | ((uint32_t)(3 * pr.y) << 16);
        }
    }
    auto fetch = [&](int64_t i, int q) {
        const float *g = src.xyz + i * row_floats;
        float *dst = ring + q * slot;
        for (int t = lane; t < row_floats; t += 32) cp_async4(dst + t, g + t);
    };
    for (int64_t piece = gwarp; piece < npieces; piece += nwarps) {
        const int64_t p0 = piece * kPiece;
        int my_i[kGroups], my_l[kGroups];
#pragma unroll
        for (int g = 0; g < kGroups; ++g) {
            const int64_t p = p0 + 32 * g + lane;
            my_i[g] = p < n ? perm[p] : 0;
            my_l[g] = p < n ? slab[p] : -1;
        }
        // the first kPairSlots - 1 frames of the piece (the valid positions
        // are a prefix of it), a copy group each
#pragma unroll
        for (int t = 0; t < kPairSlots - 1; ++t) {
            if (__shfl_sync(0xffffffffu, my_l[0], t) >= 0) fetch(__shfl_sync(0xffffffffu, my_i[0], t), t);
            cp_async_commit();
        }
        CSum acc[MW], qacc;
        float cold[MW];
        int cur = -1;
        auto flush = [&]() {
#pragma unroll
            for (int m = 0; m < MW; ++m) {
                const int f = f_base + lane + 32 * m;
                if (f < d) atomicAdd(&S[(int64_t)cur * d + f], acc[m].value());
            }
            double q = qacc.value();
            for (int off = 16; off > 0; off >>= 1) q += __shfl_xor_sync(0xffffffffu, q, off);
            if (lane == 0) atomicAdd(&Q[cur], q);
        };
#pragma unroll
        for (int g = 0; g < kGroups; ++g) {
            for (int r = 0; r < 32; ++r) {
                const int l = __shfl_sync(0xffffffffu, my_l[g], r);
                if (l < 0) break;
                // Position t + kPairSlots - 1 into the slot that frame t - 1
                // used (read by every lane before the last __syncwarp).
                const int t = 32 * g + r;
                {
                    const int tn = r + kPairSlots - 1;
                    const int gn = g + 1 < kGroups ? g + 1 : g;  // a constant once unrolled
                    int ln = -1, in = 0;
                    if (tn < 32) {
                        ln = __shfl_sync(0xffffffffu, my_l[g], tn);
                        in = __shfl_sync(0xffffffffu, my_i[g], tn);
                    } else if (g + 1 < kGroups) {
                        ln = __shfl_sync(0xffffffffu, my_l[gn], tn - 32);
                        in = __shfl_sync(0xffffffffu, my_i[gn], tn - 32);
                    }
                    if (ln >= 0) fetch(in, (t + kPairSlots - 1) % kPairSlots);
                    cp_async_commit();
                }
                cp_async_wait<kPairSlots - 1>();  // frame t's group has landed (this lane's part)
                __syncwarp();                     // ... and every lane's
                const float *xr = ring + (t % kPairSlots) * slot;
                if (l != cur) {
                    if (cur >= 0) flush();
                    cur = l;
                    qacc.reset();
#pragma unroll
                    for (int m = 0; m < MW; ++m) {
                        const int f = f_base + lane + 32 * m;
                        acc[m].reset();
                        cold[m] = f < d ? __ldg(C_old + (int64_t)l * d + f) : 0.0f;
                    }
                }
#pragma unroll
                for (int m = 0; m < MW; ++m) {
                    const int f = f_base + lane + 32 * m;
                    if (f < d) {
                        const float *a = xr + (ofs[m] & 0xFFFFu);
                        const float *b = xr + (ofs[m] >> 16);
                        const float x = pair_feature(a[0], a[1], a[2], b[0], b[1], b[2]);
                        const float t2 = x - cold[m];
                        acc[m].add(t2);
                        qacc.add(t2 * t2);
                    }
                }
                __syncwarp();
            }
        }
        if (cur >= 0) flush();
        cp_async_wait<0>();  // no copy into the ring outlives the piece
        __syncwarp();
    }
}

template <int DP, class Src>
__global__ void __launch_bounds__(256) seg_accumulate_narrow_kernel(
    const Src src, int d, const int32_t *__restrict__ perm, const int32_t *__restrict__ slab,
    int64_t n_max, const int32_t *__restrict__ n_sorted, const float *__restrict__ C_old, double *__restrict__ S,
    double *__restrict__ Q) {
    constexpr int R = 32 / DP;
    const int64_t n = min(n_max, (int64_t)*n_sorted);
    const int lane = threadIdx.x & 31;
    const int slot = lane / DP;
    const int f = lane % DP;
    const bool fvalid = f < d;
    const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t npieces = (n + kPiece - 1) / kPiece;
    for (int64_t piece = gwarp; piece < npieces; piece += nwarps) {
        const int64_t p0 = piece * kPiece;
        const int64_t p1 = min(p0 + kPiece, n);
        CSum acc, qacc;
        float cold = 0.0f;
        int cur = -1;
        for (int64_t p = p0 + slot; p < p1; p += R) {
            const int l = slab[p];
            const int64_t i = perm[p];
            if (l != cur) {
                if (cur >= 0 && fvalid) {
                    atomicAdd(&S[(int64_t)cur * d + f], acc.value());
                    atomicAdd(&Q[cur], qacc.value());
                }
                cur = l;
                acc.reset();
                qacc.reset();
                cold = fvalid ? __ldg(C_old + (int64_t)l * d + f) : 0.0f;
            }
            if (fvalid) {
                const float t = src.get(i, f) - cold;
                acc.add(t);
                qacc.add(t * t);
            }
        }
        if (cur >= 0 && fvalid) {
            atomicAdd(&S[(int64_t)cur * d + f], acc.value());
            atomicAdd(&Q[cur], qacc.value());
        }
    }
}

// One warp per cluster: new center, per-cluster inertia.
__global__ void finalize_kernel(const double *__restrict__ S, const double *__restrict__ Q,
                                const int32_t *__restrict__ counts, const float *__restrict__ C_old,
                                float *__restrict__ C_new, int d, int k, double *__restrict__ ccost,
                                int64_t *__restrict__ counts_out) {
    const int lane = threadIdx.x & 31;
    const int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (j >= k) return;
    const int cnt = counts[j];
    const float *c = C_old + j * d;
    float *m = C_new + j * d;
    if (cnt == 0) {
        for (int f = lane; f < d; f += 32) m[f] = c[f];
        if (lane == 0) ccost[j] = 0.0;
    } else {
        const double dc = (double)cnt;
        // one float64 division per center, not per element (FP64 divisions
        // are slow on this part): S_j / n_j as S_j times the reciprocal, at
        // most a float64 rounding apart before mu is rounded to float
        const double inv = 1.0 / dc;
        const double *s = S + j * d;
        double cross = 0.0, sq = 0.0;
        for (int f = lane; f < d; f += 32) {
            const float mu = (float)((double)c[f] + s[f] * inv);
            const double dl = (double)mu - (double)c[f];
            cross += dl * s[f];
            sq += dl * dl;
            m[f] = mu;
        }
        for (int off = 16; off > 0; off >>= 1) {
            cross += __shfl_xor_sync(0xffffffffu, cross, off);
            sq += __shfl_xor_sync(0xffffffffu, sq, off);
        }
        if (lane == 0) ccost[j] = Q[j] - 2.0 * cross + dc * sq;
    }
    if (counts_out && lane == 0) counts_out[j] = cnt;
}

// One warp per listed frame: its contribution (float32 deviations from the
// previous centers, as the segment sums take them) leaves the cluster of its
// first label and joins that of its exact label.
template <class Src>
__global__ void apply_flips_kernel(const Src src, int d, const float *__restrict__ C_old,
                                   const int32_t *__restrict__ flips, const int32_t *__restrict__ n_flips,
                                   int64_t max_flips, int32_t *__restrict__ labels, int32_t *__restrict__ counts,
                                   double *__restrict__ S, double *__restrict__ Q) {
    int64_t nf = *n_flips;
    if (nf > max_flips) nf = max_flips;
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nf; w += nw) {
        const int64_t frame = flips[3 * w];
        const int from = flips[3 * w + 1];
        const int to = flips[3 * w + 2];
        const float *cf = C_old + (int64_t)from * d;
        const float *ct = C_old + (int64_t)to * d;
        double qf = 0.0, qt = 0.0;
        for (int f = lane; f < d; f += 32) {
            const float xf = src.get(frame, f);
            const float tf = __fsub_rn(xf, cf[f]);
            const float tt = __fsub_rn(xf, ct[f]);
            atomicAdd(&S[(int64_t)from * d + f], -(double)tf);
            atomicAdd(&S[(int64_t)to * d + f], (double)tt);
            qf += (double)__fmul_rn(tf, tf);
            qt += (double)__fmul_rn(tt, tt);
        }
        for (int off = 16; off > 0; off >>= 1) {
            qf += __shfl_xor_sync(0xffffffffu, qf, off);
            qt += __shfl_xor_sync(0xffffffffu, qt, off);
        }
        if (lane == 0) {
            atomicAdd(&Q[from], -qf);
            atomicAdd(&Q[to], qt);
            atomicSub(&counts[from], 1);
            atomicAdd(&counts[to], 1);
            labels[frame] = to;
        }
    }
}

// Few centers and features (d <= 16 and every center's sums fit in 48 KB of
// shared memory): one pass instead of the counting sort and segment pass.
// Each thread walks a run of consecutive frames (time-ordered frames often
// share a label), sums the deviations x - c_old of each feature with a
// compensated float sum and the frame's squared deviations (one fused
// multiply-add chain) into a compensated total, as the segment kernels do,
// and adds the run's partial sums to the CTA's float64 sums in shared memory
// whenever the label changes.  The CTA adds each of its totals to global
// memory once.  Only the order of the float64 additions differs from the
// segment path.
constexpr size_t kSmallSumsBytes = 48 * 1024;
constexpr int kSmallThreads = 256;
constexpr int kSmallMaxRun = 16;

size_t small_sums_bytes(int d, int k) { return ((size_t)k * d + k) * sizeof(double) + (size_t)k * sizeof(int32_t); }

bool small_ok(int d, int k) { return d <= 16 && small_sums_bytes(d, k) <= kSmallSumsBytes; }

template <int DP>
__global__ void __launch_bounds__(kSmallThreads) small_accumulate_kernel(
    const float *__restrict__ X, int64_t n, int d, const int32_t *__restrict__ labels, int k,
    const float *__restrict__ C_old, int run, int32_t *__restrict__ counts, double *__restrict__ S,
    double *__restrict__ Q, uint32_t *err) {
    extern __shared__ double small_sums[];
    double *S_s = small_sums;
    double *Q_s = S_s + (size_t)k * d;
    int32_t *c_s = reinterpret_cast<int32_t *>(Q_s + k);
    for (int e = threadIdx.x; e < k * d + k; e += blockDim.x) small_sums[e] = 0.0;
    for (int e = threadIdx.x; e < k; e += blockDim.x) c_s[e] = 0;
    __syncthreads();
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nt = (int64_t)gridDim.x * blockDim.x;
    for (int64_t r0 = tid * run; r0 < n; r0 += nt * run) {
        const int64_t r1 = min(r0 + (int64_t)run, n);
        CSum acc[DP], qacc;
        float cold[DP];
        int cur = -1, cnt = 0;
        auto flush = [&]() {
#pragma unroll
            for (int f = 0; f < DP; ++f)
                if (f < d) atomicAdd(&S_s[cur * d + f], acc[f].value());
            atomicAdd(&Q_s[cur], qacc.value());
            atomicAdd(&c_s[cur], cnt);
        };
        for (int64_t i = r0; i < r1; ++i) {
            const int j = labels[i];
            if (j < 0 || j >= k) {
                atomicOr(err, (uint32_t)kDevBadLabel);
                continue;
            }
            if (j != cur) {
                if (cur >= 0) flush();
                cur = j;
                cnt = 0;
                qacc.reset();
#pragma unroll
                for (int f = 0; f < DP; ++f) {
                    acc[f].reset();
                    cold[f] = f < d ? __ldg(C_old + (int64_t)j * d + f) : 0.0f;
                }
            }
            float q = 0.0f;
#pragma unroll
            for (int f = 0; f < DP; ++f) {
                if (f < d) {
                    const float t = __fsub_rn(__ldg(X + i * d + f), cold[f]);
                    acc[f].add(t);
                    q = __fmaf_rn(t, t, q);
                }
            }
            qacc.add(q);
            ++cnt;
        }
        if (cur >= 0) flush();
    }
    __syncthreads();
    for (int e = threadIdx.x; e < k * d; e += blockDim.x)
        if (S_s[e] != 0.0) atomicAdd(&S[e], S_s[e]);
    for (int e = threadIdx.x; e < k; e += blockDim.x) {
        if (c_s[e]) {
            atomicAdd(&Q[e], Q_s[e]);
            atomicAdd(&counts[e], c_s[e]);
        }
    }
}

__global__ void add_counts_kernel(const int32_t *__restrict__ counts, int k, int32_t *__restrict__ total) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < k; j += gridDim.x * blockDim.x) total[j] += counts[j];
}

// Single CTA, fixed summation tree: the same inputs give the same cost.
__global__ void __launch_bounds__(1024) reduce_cost_kernel(const double *__restrict__ ccost, int k,
                                                            double *__restrict__ cost) {
    __shared__ double part[1024];
    double s = 0.0;
    for (int j = threadIdx.x; j < k; j += blockDim.x) s += ccost[j];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = blockDim.x >> 1; off > 0; off >>= 1) {
        if (threadIdx.x < (unsigned)off) part[threadIdx.x] += part[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) *cost = part[0];
}

PairRows pair_rows_of(const PairSrc &ps, int d) {
    return PairRows{ps.xyz, reinterpret_cast<const int2 *>(ps.pairs), ps.n_atoms, d};
}

unsigned grid_for(int64_t work, int threads, int per_sm) {
    int64_t g = (work + threads - 1) / threads;
    int64_t cap = (int64_t)num_sms() * per_sm;
    if (g > cap) g = cap;
    return (unsigned)(g < 1 ? 1 : g);
}

template <int MW, class Src>
void launch_wide(const Src &X, int64_t n, int d, const UpdateWs &u, int k, const float *C_old, unsigned g,
                 cudaStream_t s) {
    for (int f_base = 0; f_base < d; f_base += 32 * MW)
        seg_accumulate_wide_kernel<MW, Src><<<g, 256, 0, s>>>(X, d, f_base, u.perm, u.slab, n, u.offsets + k,
                                                              C_old, u.S, u.Q);
}

template <int DP, class Src>
void launch_narrow(const Src &X, int64_t n, int d, const UpdateWs &u, int k, const float *C_old, unsigned g,
                   cudaStream_t s) {
    seg_accumulate_narrow_kernel<DP, Src><<<g, 256, 0, s>>>(X, d, u.perm, u.slab, n, u.offsets + k, C_old, u.S,
                                                            u.Q);
}

template <int MW, class Src>
bool try_wide(int mw, const Src &X, int64_t n, int d, const UpdateWs &u, int k, const float *C_old, unsigned g,
              cudaStream_t s) {
    if (mw > MW) return false;
    launch_wide<MW>(X, n, d, u, k, C_old, g, s);
    return true;
}

template <int MW, int RING>
int launch_bulk_ring(const float *X, int64_t n, int d, const UpdateWs &u, int k, const float *C_old, uint32_t *err,
                     cudaStream_t s, int seg_per_sm) {
    const size_t smem = bulk_smem_bytes(MW, RING);
    // Per device (the shared-memory opt-in holds per device), cached so that
    // no attribute call happens while a stream is being captured.
    static int per_sm_dev[kDeviceSlots] = {};
    const int dev = current_device();
    int per_sm = dev >= 0 && dev < kDeviceSlots ? per_sm_dev[dev] : 0;
    if (per_sm <= 0) {
        KM_CUDA(cudaFuncSetAttribute(seg_accumulate_bulk_kernel<MW, RING>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(232448)));
        int v = 0;
        KM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, seg_accumulate_bulk_kernel<MW, RING>,
                                                              kBulkWarps * 32, smem));
        per_sm = v > 0 ? v : 1;
        if (dev >= 0 && dev < kDeviceSlots) per_sm_dev[dev] = per_sm;
    }
    const int64_t npieces = (n + kPiece - 1) / kPiece;
    int64_t g = (npieces + kBulkWarps - 1) / kBulkWarps;
    const int64_t cap = (int64_t)num_sms() * (seg_per_sm > 0 && seg_per_sm < per_sm ? seg_per_sm : per_sm);
    if (g > cap) g = cap;
    seg_accumulate_bulk_kernel<MW, RING><<<(unsigned)(g < 1 ? 1 : g), kBulkWarps * 32, smem, s>>>(
        X, d, u.perm, u.slab, n, u.offsets + k, C_old, u.S, u.Q, err);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

// One CTA per SM (room for another kernel beside it) keeps twice the rows in
// flight per warp when they fit in shared memory.
template <int MW>
int launch_bulk(const float *X, int64_t n, int d, const UpdateWs &u, int k, const float *C_old, uint32_t *err,
                cudaStream_t s, int seg_per_sm) {
    if (seg_per_sm == 1 && bulk_smem_bytes(MW, 2 * kRing) <= 227 * 1024)
        return launch_bulk_ring<MW, 2 * kRing>(X, n, d, u, k, C_old, err, s, seg_per_sm);
    return launch_bulk_ring<MW, kRing>(X, n, d, u, k, C_old, err, s, seg_per_sm);
}

int launch_segments_bulk(const float *X, int64_t n, int d, const UpdateWs &u, int k, const float *C_old,
                         uint32_t *err, cudaStream_t s, int seg_per_sm) {
    const int mw = (d + 31) / 32;
    switch (mw) {
        case 1: return launch_bulk<1>(X, n, d, u, k, C_old, err, s, seg_per_sm);
        case 2: return launch_bulk<2>(X, n, d, u, k, C_old, err, s, seg_per_sm);
        case 3: return launch_bulk<3>(X, n, d, u, k, C_old, err, s, seg_per_sm);
        case 4: return launch_bulk<4>(X, n, d, u, k, C_old, err, s, seg_per_sm);
        case 5: case 6: return launch_bulk<6>(X, n, d, u, k, C_old, err, s, seg_per_sm);
        case 7: case 8: return launch_bulk<8>(X, n, d, u, k, C_old, err, s, seg_per_sm);
        case 9: case 10: case 11: case 12: return launch_bulk<12>(X, n, d, u, k, C_old, err, s, seg_per_sm);
        case 13: case 14: case 15: case 16: case 17: return launch_bulk<17>(X, n, d, u, k, C_old, err, s, seg_per_sm);
        case 18: case 19: case 20: case 21: case 22: case 23: case 24: return launch_bulk<24>(X, n, d, u, k, C_old, err, s, seg_per_sm);
        default: return launch_bulk<32>(X, n, d, u, k, C_old, err, s, seg_per_sm);
    }
}

bool bulk_ok(const float *X, int d) {
    return d >= 32 && d <= 1024 && (d % 4) == 0 && (reinterpret_cast<uintptr_t>(X) % 16) == 0;
}

template <class Src>
int launch_segments(const Src &X, int64_t n, int d, const UpdateWs &u, int k, const float *C_old, unsigned g,
                    cudaStream_t s) {
    if (d >= 32) {
        const int mw = (d + 31) / 32;
        const bool ok = try_wide<1>(mw, X, n, d, u, k, C_old, g, s) || try_wide<2>(mw, X, n, d, u, k, C_old, g, s) ||
                        try_wide<3>(mw, X, n, d, u, k, C_old, g, s) || try_wide<4>(mw, X, n, d, u, k, C_old, g, s) ||
                        try_wide<6>(mw, X, n, d, u, k, C_old, g, s) || try_wide<8>(mw, X, n, d, u, k, C_old, g, s) ||
                        try_wide<12>(mw, X, n, d, u, k, C_old, g, s) || try_wide<17>(mw, X, n, d, u, k, C_old, g, s) ||
                        try_wide<24>(mw, X, n, d, u, k, C_old, g, s) || try_wide<32>(mw, X, n, d, u, k, C_old, g, s);
        if (!ok) launch_wide<32>(X, n, d, u, k, C_old, g, s);  // d > 1024: slices of 1024 features
    } else if (d > 16) {
        launch_narrow<32>(X, n, d, u, k, C_old, g, s);
    } else if (d > 8) {
        launch_narrow<16>(X, n, d, u, k, C_old, g, s);
    } else if (d > 4) {
        launch_narrow<8>(X, n, d, u, k, C_old, g, s);
    } else if (d > 2) {
        launch_narrow<4>(X, n, d, u, k, C_old, g, s);
    } else if (d > 1) {
        launch_narrow<2>(X, n, d, u, k, C_old, g, s);
    } else {
        launch_narrow<1>(X, n, d, u, k, C_old, g, s);
    }
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

template <int MW>
int launch_pairs_mw(const PairRows &src, int64_t n, int d, const UpdateWs &u, int k, const float *C_old,
                    cudaStream_t s) {
    const size_t smem = pair_seg_smem(src.n_atoms);
    // resident CTAs per SM for this slot size (the grid walks its pieces in
    // a fixed order per warp, so it is sized to what is resident at once)
    static std::mutex mu;
    static std::map<std::pair<int, size_t>, int> per_sm_of;  // (device, shared memory) -> CTAs per SM
    int per_sm = 0;
    {
        const auto key = std::make_pair(current_device(), smem);
        std::lock_guard<std::mutex> lk(mu);
        auto it = per_sm_of.find(key);
        if (it == per_sm_of.end()) {
            int v = 0;
            KM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, seg_accumulate_pairs_kernel<MW>, 256, smem));
            it = per_sm_of.emplace(key, v > 0 ? v : 1).first;
        }
        per_sm = it->second;
    }
    const int64_t npieces = (n + kPiece - 1) / kPiece;
    const unsigned g = grid_for(npieces * 32, 256, per_sm);
    for (int f_base = 0; f_base < d; f_base += 32 * MW)
        seg_accumulate_pairs_kernel<MW><<<g, 256, smem, s>>>(src, d, f_base, u.perm, u.slab, n, u.offsets + k,
                                                              C_old, u.S, u.Q);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

int launch_segments_pairs(const PairRows &src, int64_t n, int d, const UpdateWs &u, int k, const float *C_old,
                          cudaStream_t s) {
    const int mw = (d + 31) / 32;
    if (mw <= 1) return launch_pairs_mw<1>(src, n, d, u, k, C_old, s);
    if (mw <= 2) return launch_pairs_mw<2>(src, n, d, u, k, C_old, s);
    if (mw <= 4) return launch_pairs_mw<4>(src, n, d, u, k, C_old, s);
    if (mw <= 8) return launch_pairs_mw<8>(src, n, d, u, k, C_old, s);
    if (mw <= 12) return launch_pairs_mw<12>(src, n, d, u, k, C_old, s);
    if (mw <= 17) return launch_pairs_mw<17>(src, n, d, u, k, C_old, s);
    if (mw <= 24) return launch_pairs_mw<24>(src, n, d, u, k, C_old, s);
    return launch_pairs_mw<32>(src, n, d, u, k, C_old, s);  // d > 1024: slices of 1024 features
}

}  // namespace

size_t update_ws_size(int64_t n, int d, int k) {
    size_t b = 0;
    carve(nullptr, n, d, k, &b);
    return b;
}

int32_t *update_counts(void *ws, int64_t n, int d, int k) { return carve(ws, n, d, k, nullptr).counts; }

bool update_counts_from_labels(int d, int k, const PairSrc *ps) { return ps || !small_ok(d, k); }

int launch_update_accumulate(const float *X, int64_t n, int d, const int32_t *labels, int k, const float *C_old,
                             uint32_t *err, void *ws, cudaStream_t s, int seg_per_sm, const PairSrc *ps,
                             bool counted) {
    UpdateWs u = carve(ws, n, d, k, nullptr);
    if (counted && !update_counts_from_labels(d, k, ps)) {
        set_error("precounted members only on the counting-sort path of the update");
        return KM_ERR_UNSUPPORTED;
    }
    if (!counted) KM_CUDA(cudaMemsetAsync(u.counts, 0, sizeof(int32_t) * k, s));
    KM_CUDA(cudaMemsetAsync(u.S, 0, sizeof(double) * (size_t)k * d, s));
    KM_CUDA(cudaMemsetAsync(u.Q, 0, sizeof(double) * k, s));
    if (n > 0 && !ps && small_ok(d, k)) {
        const int dp = d <= 1 ? 1 : d <= 2 ? 2 : d <= 4 ? 4 : d <= 8 ? 8 : 16;
        // one frame per thread while the frames fill 8 CTAs of every SM, runs
        // of up to kSmallMaxRun frames beyond that
        const int64_t slots = (int64_t)num_sms() * 8 * kSmallThreads;
        const int run = (int)std::min<int64_t>(kSmallMaxRun, std::max<int64_t>(1, (n + slots - 1) / slots));
        const unsigned g = grid_for((n + run - 1) / run, kSmallThreads, 8);
        const size_t smem = small_sums_bytes(d, k);
        switch (dp) {
#define KM_SMALL(DP)                                                                                          \
    case DP:                                                                                                  \
        small_accumulate_kernel<DP><<<g, kSmallThreads, smem, s>>>(X, n, d, labels, k, C_old, run, u.counts, \
                                                                   u.S, u.Q, err);                           \
        break;
            KM_SMALL(1) KM_SMALL(2) KM_SMALL(4) KM_SMALL(8) KM_SMALL(16)
#undef KM_SMALL
        }
        KM_CUDA(cudaGetLastError());
        return KM_OK;
    }
    if (n > 0 && !counted) {
        count_labels_kernel<<<grid_for(n, 256, 8), 256, 0, s>>>(labels, n, k, u.counts, err);
        KM_CUDA(cudaGetLastError());
    }
    scan_counts_kernel<<<1, 1024, 0, s>>>(u.counts, k, u.offsets, u.cursor);
    KM_CUDA(cudaGetLastError());
    if (n > 0) {
        scatter_kernel<<<grid_for(n, 256, 8), 256, 0, s>>>(labels, n, k, u.cursor, u.perm, u.slab);
        KM_CUDA(cudaGetLastError());
        if (ps) {
            // pair features: computed where the segment sums read them
            if (ps->n_atoms <= kPairMaxAtoms) {
                KM_TRY(launch_segments_pairs(pair_rows_of(*ps, d), n, d, u, k, C_old, s));
            } else {
                const int64_t npieces = (n + kPiece - 1) / kPiece;
                const unsigned g = grid_for(npieces * 32, 256, 8);
                KM_TRY(launch_segments(pair_rows_of(*ps, d), n, d, u, k, C_old, g, s));
            }
        } else if (bulk_ok(X, d)) {
            KM_TRY(launch_segments_bulk(X, n, d, u, k, C_old, err, s, seg_per_sm));
        } else {
            const int64_t npieces = (n + kPiece - 1) / kPiece;
            const unsigned g = grid_for(npieces * 32, 256, 8);
            KM_TRY(launch_segments(DenseRows{X, d}, n, d, u, k, C_old, g, s));
        }
    }
    return KM_OK;
}

int launch_update_finish(int64_t n, int d, int k, const float *C_old, float *C_new, int64_t *counts_out,
                         double *cost, void *ws, cudaStream_t s) {
    UpdateWs u = carve(ws, n, d, k, nullptr);
    finalize_kernel<<<(unsigned)(((int64_t)k * 32 + 255) / 256), 256, 0, s>>>(
        u.S, u.Q, u.counts, C_old, C_new, d, k, u.ccost, counts_out);
    KM_CUDA(cudaGetLastError());
    reduce_cost_kernel<<<1, 1024, 0, s>>>(u.ccost, k, cost);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

int launch_apply_flips(const float *X, int64_t n, int d, int k, const float *C_old, const FlipList &fl,
                       int32_t *labels, void *ws, cudaStream_t s, const PairSrc *ps) {
    if (fl.cap == 0) return KM_OK;
    UpdateWs u = carve(ws, n, d, k, nullptr);
    const unsigned g = grid_for(fl.cap * 32, 256, 4);
    if (ps)
        apply_flips_kernel<<<g, 256, 0, s>>>(pair_rows_of(*ps, d), d, C_old, fl.rows, fl.count, fl.cap, labels,
                                              u.counts, u.S, u.Q);
    else
        apply_flips_kernel<<<g, 256, 0, s>>>(DenseRows{X, d}, d, C_old, fl.rows, fl.count, fl.cap, labels, u.counts,
                                              u.S, u.Q);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

int launch_update(const float *X, int64_t n, int d, const int32_t *labels, int k,
                  const float *C_old, float *C_new, int64_t *counts_out, double *cost,
                  uint32_t *err, void *ws, cudaStream_t s, const PairSrc *ps) {
    KM_TRY(launch_update_accumulate(X, n, d, labels, k, C_old, err, ws, s, 0, ps));
    return launch_update_finish(n, d, k, C_old, C_new, counts_out, cost, ws, s);
}

int launch_update_parts_begin(int64_t n, int d, int k, void *ws, cudaStream_t s) {
    UpdateWs u = carve(ws, n, d, k, nullptr);
    KM_CUDA(cudaMemsetAsync(u.total, 0, sizeof(int32_t) * k, s));
    KM_CUDA(cudaMemsetAsync(u.S, 0, sizeof(double) * (size_t)k * d, s));
    KM_CUDA(cudaMemsetAsync(u.Q, 0, sizeof(double) * k, s));
    return KM_OK;
}

int launch_update_part(const float *X, int64_t n, int d, const int32_t *labels, int64_t rows, int k,
                       const float *C_old, uint32_t *err, void *ws, cudaStream_t s) {
    if (rows == 0) return KM_OK;
    UpdateWs u = carve(ws, n, d, k, nullptr);
    // The counting sort and the segment sums of these rows, into the totals;
    // launch_update_accumulate without its clearing of the sums.
    KM_CUDA(cudaMemsetAsync(u.counts, 0, sizeof(int32_t) * k, s));
    count_labels_kernel<<<grid_for(rows, 256, 8), 256, 0, s>>>(labels, rows, k, u.counts, err);
    KM_CUDA(cudaGetLastError());
    scan_counts_kernel<<<1, 1024, 0, s>>>(u.counts, k, u.offsets, u.cursor);
    KM_CUDA(cudaGetLastError());
    scatter_kernel<<<grid_for(rows, 256, 8), 256, 0, s>>>(labels, rows, k, u.cursor, u.perm, u.slab);
    KM_CUDA(cudaGetLastError());
    if (bulk_ok(X, d)) {
        KM_TRY(launch_segments_bulk(X, rows, d, u, k, C_old, err, s, 0));
    } else {
        const int64_t npieces = (rows + kPiece - 1) / kPiece;
        KM_TRY(launch_segments(DenseRows{X, d}, rows, d, u, k, C_old, grid_for(npieces * 32, 256, 8), s));
    }
    add_counts_kernel<<<(unsigned)((k + 255) / 256), 256, 0, s>>>(u.counts, k, u.total);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

int launch_update_parts_finish(int64_t n, int d, int k, const float *C_old, float *C_new, double *cost, void *ws,
                               cudaStream_t s) {
    UpdateWs u = carve(ws, n, d, k, nullptr);
    KM_CUDA(cudaMemcpyAsync(u.counts, u.total, sizeof(int32_t) * k, cudaMemcpyDeviceToDevice, s));
    return launch_update_finish(n, d, k, C_old, C_new, nullptr, cost, ws, s);
}

}  // namespace km

// ---------------------------------------------------------------------------
// km_update_noalloc: the centroid update without a caller workspace.
//
// Some callers cannot hand out device memory: a plugin running inside a host
// program that owns every device allocation (an MD engine or a serving
// framework with its own memory pool and budget), or code that must not call
// cudaMalloc because that call can synchronise the whole device in the middle
// of a latency-sensitive loop.  This entry point uses a fixed scratch array
// that is part of the library image instead.  The array costs
// kNoAllocScratchBytes of device memory on every GPU that loads the library,
// for as long as the process runs.
// ---------------------------------------------------------------------------
namespace km {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;  // 32 MiB

static __device__ __align__(256) unsigned char g_update_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void *g_scratch_ptr[kMaxDevices] = {};
// One lock per device, held by km_update_noalloc from its first launch until
// its stream has drained: calls on one device share that device's copy of
// the scratch array, so they run one at a time; calls on different devices
// use different copies and do not wait for each other.
std::mutex g_noalloc_call_mutex[kMaxDevices];

// Device address of g_update_scratch on the current device.  In host code the
// array's name is only a stand-in, so the address is looked up once per
// device (with that device current) and cached.  *dev_out receives the
// device ordinal.
int scratch_address(void **out, int *dev_out) {
    int dev = 0;
    KM_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("device ordinal %d is beyond the %d devices this library tracks", dev, kMaxDevices);
        return KM_ERR_UNSUPPORTED;
    }
    *dev_out = dev;
    std::lock_guard<std::mutex> lk(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_update_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_update_scratch)");
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return KM_OK;
}

}  // namespace
}  // namespace km

extern "C" size_t km_update_noalloc_max_bytes(void) { return km::kNoAllocScratchBytes; }

extern "C" int km_update_noalloc(const float *X, int64_t n, int32_t d, const int32_t *labels, int32_t k,
                                 const float *C_old, float *C_new, int64_t *counts, double *cost,
                                 void *stream) {
    using namespace km;
    KM_TRY(check_shape(n, d, k));
    if ((n > 0 && (!X || !labels)) || !C_old || !C_new || !cost) {
        set_error("X, labels, C_old, C_new and cost must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    if (C_old == C_new) {
        set_error("C_new must not alias C_old");
        return KM_ERR_BAD_SHAPE;
    }
    // Scratch layout: the workspace of the update followed by one error word.
    const size_t need = update_ws_size(n, d, k) + 256;
    if (need > kNoAllocScratchBytes) {
        set_error("km_update_noalloc needs %zu bytes of scratch for n=%lld, d=%d, k=%d; its fixed array "
                  "holds %zu (8 n + 8 k d + 32 k bytes plus about 2.5 KB of alignment must fit; "
                  "km_update_workspace_size gives the exact figure); use km_update with a workspace",
                  need, (long long)n, d, k, kNoAllocScratchBytes);
        return KM_ERR_WORKSPACE;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // Every call reads the device error word back and synchronises `stream`,
    // which a stream capture does not allow: refuse before enqueuing anything.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t ce = cudaStreamIsCapturing(s, &cap);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamIsCapturing");
    if (cap != cudaStreamCaptureStatusNone) {
        set_error("km_update_noalloc cannot run on a stream that is being captured (it synchronises the stream)");
        return KM_ERR_UNSUPPORTED;
    }
    void *scratch = nullptr;
    int dev = 0;
    KM_TRY(scratch_address(&scratch, &dev));
    uint32_t *err = reinterpret_cast<uint32_t *>(static_cast<char *>(scratch) + update_ws_size(n, d, k));
    std::lock_guard<std::mutex> call_lock(g_noalloc_call_mutex[dev]);
    // The array keeps the previous call's contents: the error word is cleared
    // here, and launch_update clears its own counters and sums.
    ce = cudaMemsetAsync(err, 0, sizeof(uint32_t), s);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemsetAsync(error word)");
    int rc = launch_update(X, n, d, labels, k, C_old, C_new, counts, cost, err, scratch, s);
    uint32_t e = 0;
    if (rc == KM_OK) {
        ce = cudaMemcpyAsync(&e, err, sizeof(e), cudaMemcpyDeviceToHost, s);
        if (ce != cudaSuccess) rc = cuda_fail(ce, "cudaMemcpyAsync(error word)");
    }
    // drained before the lock is released, also after a failed launch
    ce = cudaStreamSynchronize(s);
    if (rc != KM_OK) return rc;
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamSynchronize");
    // Every bit of the error word maps to a status, as in km_update: a label
    // out of range, or a device-side wait of the segment sums that ran out.
    return device_error_status(e | take_fake_device_error());
}

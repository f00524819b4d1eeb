// assign_tc.cu -- kernel (b): nearest-center assignment on the tcgen05
// tensor cores (FP16 operands, FP32 accumulation), followed by an exact FP32
// recheck (kernel (b'), assign_fp32.cu) of every frame whose nearest centers
// are not separated by the derived error bound.  The resulting labels equal
// those of the exact FP32 kernel bit for bit.
//
// Reference: ClusterModel(centers, 'euclidean').transform(X),
// pyemma/coordinates/clustering/interface.py:157-167 (and the assignment step
// inside KMeans.fit, kmeans.py:253).
//
// Data flow
//   prep: x' = x - m and c' = c - m in float32 (m = the mean of the centers;
//         squared distances are translation invariant), multiplied by a power
//         of two s (chosen so that s max ||c'|| lies in (2^6, 2^7]) and
//         rounded to FP16.  Rows are padded with zeros to kp = 64 ceil((d+2)/64)
//         columns; columns d and d+1 carry 1 for frames and the FP16 hi/lo
//         split of -||c_hat||^2/2 for centers, so the accumulator holds
//         a_j = x_hat.c_hat_j - ||c_hat_j||^2/2 and
//         v_j = ||x_hat||^2 - 2 a_j = ||x_hat - c_hat_j||^2 (scaled by s^2).
//   main: persistent CTA per SM.  A frame tile (128 frames x kp) stays in
//         shared memory while center tiles (BN x kp) stream through a TMA
//         ring; one thread issues tcgen05.mma (M=128, N=BN, K=16) into one of
//         two TMEM accumulators; four epilogue warps read them with
//         tcgen05.ld.  Per frame the epilogue keeps the best a_j and, from the
//         bound, the smallest a a center must reach to stay a possible
//         argmin; a branch-free max over each 32-column chunk skips chunks
//         below that threshold, and the few centers above it go into a list
//         of L (overflow -> exact recheck over all centers).
//   decision: the bound below gives, for each listed center, an interval
//         [lo_j(v_j), hi_j(v_j)] holding the exact float32 distance D_j.  With
//         H = min_j hi_j, center j can be the exact argmin only if lo_j <= H.
//         One candidate: final label.  2..L candidates: exact recheck of
//         those.  A full list whose last entry (with the largest center norm)
//         still passes, or a non-finite value: exact recheck over all centers.
//
// Bound, in unscaled units (u = 2^-24, sx >= ||x'||, sc_j >= ||c'_j||, and
// hx >= ||x_hat/s - x'||, hc_j >= ||c_hat_j/s - c'_j|| the exact norms of the
// FP16 rounding errors, measured when the operands are made):
//   | ||x_hat - c_hat||/s - ||x - c|| | <= R_j = hx + hc_j + 2^-23 (sx + sc_j)
//   | v_j/s^2 - ||x_hat - c_hat||^2/s^2 | <= E_j = e (sx + sc_j)^2
//        e covers the tensor-core accumulation (an error of 2^-21 per 16-term
//        MMA block, four times one truncation to FP32), the hi/lo split of the
//        center norm, the rounding of ||x_hat||^2 and of v.
//   | D - ||x - c||^2 | <= g ||x - c||^2,  g = (d + 2) u / (1 - (d + 2) u)
// so lo_j(v) = (1-g) max(sqrt(max(v-E_j, 0)) - R_j, 0)^2 and
//    hi_j(v) = (1+g) (sqrt(v+E_j) + R_j)^2, evaluated with directed rounding.
#include <cuda.h>

#include <algorithm>

#include "km_common.cuh"
#include "km_internal.h"

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include <cmath>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>
#include <utility>
#include <vector>

namespace km {

namespace {

constexpr int kBM = 128;          // frames per tile (UMMA M)
constexpr int kKC = 64;           // fp16 elements per K chunk (128 B, one SW128 row)
constexpr int kL = TC_CANDIDATES; // candidates kept per frame (registers)
constexpr int kThreadsTC = 192;   // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue
constexpr int kMaxNkc = 10;       // resident A tile up to kp = 640
constexpr int kSmemLimit = 232448;
constexpr int kABytesPerChunk = kBM * kKC * 2;  // 16 KB

// Scalars shared by the prep kernels and the main kernel (uint32 words).
enum ScalarSlot { kScale = 0, kInvScale2 = 1, kScaleMax = 2, kCmax = 3, kHcMax = 4, kNumScalars = 8 };

struct TcParams {
    int64_t n;       // one past the last frame of this launch
    int64_t frame0;  // its first frame (frames [frame0, n) of the operand rows)
    int32_t *label_counts;  // nullable: each frame's tensor-core label is counted here
    int k;
    int d;
    int kp;
    int nkc;
    int ksteps_total;  // 16-wide K steps holding data (ceil((d+2)/16))
    int nbst;          // B stages per center tile (64 K columns each): ceil(ksteps_total / 4)
    int bn;
    int stages;
    int stream_a;  // 1: A chunks travel with the B stages instead of staying resident (large d)
    int bf16;      // 1: BF16 operands instead of FP16
    int n_ctiles;
    uint32_t tmem_cols;
    float e_coef;
    float g_lo;   // 1 - g, deflated
    float g_hi;   // 1 + g, inflated
    float g_ratio;  // sqrt(g_hi / g_lo), inflated
    const float4 *xnorm;
    const float2 *cnorm;
    const float *chn;  // FP8: -||c~_j||^2 / 2 per center
    const uint32_t *scal;
    int32_t *labels;
    int32_t *rc_frames;
    int32_t *pair_center;
    unsigned long long *rc_keys;
    int32_t *rc_best;
    int64_t *rc_pairs;
    float *pair_lo;
    int32_t *full_frames;
    unsigned long long *full_keys;
    int32_t *counters;
    uint32_t *err;
    float *dump;  // optional n x k distances (diagnostics)
    unsigned long long *wait_cycles;  // optional per-role wait counters (diagnostics), WaitSlot order
    // Seed of each frame's running best (16-bit operands, short rows): the
    // operand rows of the frames and centers, or null for no seed, and the
    // rounding factor of a float32 dot product over kp columns.
    const void *seed_xh;
    const void *seed_ch;
    float seed_coef;
};

// Diagnostic counters: SM cycles each role spent waiting (summed over CTAs).
enum WaitSlot {
    kWaitProdB = 0,     // producer: B stage free
    kWaitProdA = 1,     // producer: A chunk free
    kWaitMmaB = 2,      // MMA: B stage loaded
    kWaitMmaA = 3,      // MMA: A chunk loaded
    kWaitMmaAcc = 4,    // MMA: accumulator drained by the epilogue
    kWaitEpiAcc = 5,    // epilogue: accumulator ready
    kEpiTotal = 6,      // epilogue: all cycles of its loop
    kMmaTotal = 7,      // MMA: all cycles of its loop
    kNumWaitSlots = 8
};

// ---------------------------------------------------------------------------
// PTX wrappers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// One lane of the converged warp (the same lane every time).
__device__ __forceinline__ bool elect_one() {
    uint32_t pred = 0;
    asm volatile(
        "{\n\t.reg .pred P;\n\t"
        "elect.sync _|P, 0xffffffff;\n\t"
        "selp.u32 %0, 1, 0, P;\n\t}"
        : "=r"(pred));
    return pred != 0;
}

// Waits for the phase of the given parity; false after kWaitLimitNs.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t spin = 1;; ++spin) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((spin & 255u) == 0 && globaltimer_ns() - t0 > kWaitLimitNs) return false;
    }
}

// mbar_wait that adds the cycles it spent to *acc when acc is non-null.
__device__ __forceinline__ bool mbar_wait_timed(uint64_t *bar, uint32_t parity, unsigned long long *acc) {
    if (!acc) return mbar_wait(bar, parity);
    const long long t0 = clock64();
    const bool ok = mbar_wait(bar, parity);
    *acc += (unsigned long long)(clock64() - t0);
    return ok;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *tm, int x, int y,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t *holder, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(holder)),
                 "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// FP8 (e4m3 x e4m3 -> F32): the same operand layout, 32 elements (32 bytes)
// per K step.
__device__ __forceinline__ void mma_f8(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

// ---- CTA pairs (cluster of 2, tcgen05 cta_group::2) ----
__device__ __forceinline__ uint32_t cluster_ctarank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// Address of the same shared-memory offset in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t mapa_shared(uint32_t addr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}

// Every thread of both CTAs.
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Arrive on a barrier of either CTA of the pair.  The default (CTA-scope)
// release: the arrive only has to follow the thread's completed tcgen05.ld of
// the accumulator (ordered by tcgen05.fence::before_thread_sync), not its
// global stores, which a cluster-scope release would wait for.
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t cluster_addr) {
    asm volatile("mbarrier.arrive.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr) : "memory");
}

// Wait on a local barrier that threads of the peer CTA arrive on.
__device__ __forceinline__ bool mbar_try_wait_cluster(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_cluster(uint64_t *bar, uint32_t parity) {
    if (mbar_try_wait_cluster(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t spin = 1;; ++spin) {
        if (mbar_try_wait_cluster(bar, parity)) return true;
        if ((spin & 255u) == 0 && globaltimer_ns() - t0 > kWaitLimitNs) return false;
    }
}

__device__ __forceinline__ bool mbar_wait_cluster_timed(uint64_t *bar, uint32_t parity, unsigned long long *acc) {
    if (!acc) return mbar_wait_cluster(bar, parity);
    const long long t0 = clock64();
    const bool ok = mbar_wait_cluster(bar, parity);
    *acc += (unsigned long long)(clock64() - t0);
    return ok;
}

// TMA load into this CTA's shared memory whose completion is counted on the
// barrier at `bar_cluster_addr` (the leader CTA's).
__device__ __forceinline__ void tma_load_2d_pair(void *dst, const CUtensorMap *tm, int x, int y,
                                                 uint32_t bar_cluster_addr) {
    asm volatile(
        "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
        "%3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(bar_cluster_addr)
        : "memory");
}

__device__ __forceinline__ void tmem_alloc_pair(uint32_t *holder, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(holder)),
                 "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tmem_relinquish_pair() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc_pair(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_f16_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                              uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_f8_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                             uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

template <bool F8>
__device__ __forceinline__ void mma_op(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
    if constexpr (F8)
        mma_f8(d_tmem, adesc, bdesc, idesc, accumulate);
    else
        mma_f16(d_tmem, adesc, bdesc, idesc, accumulate);
}

template <bool F8>
__device__ __forceinline__ void mma_op_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
    if constexpr (F8)
        mma_f8_pair(d_tmem, adesc, bdesc, idesc, accumulate);
    else
        mma_f16_pair(d_tmem, adesc, bdesc, idesc, accumulate);
}

// Arrive on the barrier at this offset in both CTAs of the pair once the
// issuing thread's earlier MMAs are complete.
__device__ __forceinline__ void mma_commit_pair(uint64_t *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
            smem_u32(bar)),
        "h"((unsigned short)3)
        : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
          "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
          "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}

// max of three floats in one instruction (PTX max.f32 with three inputs,
// sm_100 and later): NaN inputs are ignored as by fmaxf.
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

__device__ __forceinline__ void tmem_wait_ld() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major operand in the 128-byte swizzle
// layout written by TMA (8-row atoms of 128 B, atoms 1024 B apart).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t desc = 0;
    desc |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
    desc |= (uint64_t)1 << 16;                    // leading byte offset (unused for SW128 K-major)
    desc |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset: 8 rows x 128 B
    desc |= (uint64_t)1 << 46;                    // descriptor version
    desc |= (uint64_t)2 << 61;                    // 128-byte swizzle
    return desc;
}

// Instruction descriptor of kind::f16: FP16 x FP16 (or BF16 x BF16) -> F32,
// both K-major.  The operand-type code 0 is E4M3 under kind::f8f6f4, so the
// FP16 descriptor also serves the FP8 MMA.
__host__ __device__ constexpr uint32_t make_idesc(int M, int N, bool bf16 = false) {
    return (1u << 4) | (bf16 ? ((1u << 7) | (1u << 10)) : 0u) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

// The 16-bit operand type of the tensor-core pass.
template <typename T>
struct Op16;
template <>
struct Op16<__half> {
    using T2 = __half2;
    static __device__ __forceinline__ T2 pack(float a, float b) { return __floats2half2_rn(a, b); }
    static __device__ __forceinline__ float lo(T2 v) { return __low2float(v); }
    static __device__ __forceinline__ float hi(T2 v) { return __high2float(v); }
    static __device__ __forceinline__ __half one(float v) { return __float2half_rn(v); }
    static __device__ __forceinline__ float to_float(__half v) { return __half2float(v); }
    static constexpr double kMax = 65504.0;
};
template <>
struct Op16<__nv_bfloat16> {
    using T2 = __nv_bfloat162;
    static __device__ __forceinline__ T2 pack(float a, float b) { return __floats2bfloat162_rn(a, b); }
    static __device__ __forceinline__ float lo(T2 v) { return __low2float(v); }
    static __device__ __forceinline__ float hi(T2 v) { return __high2float(v); }
    static __device__ __forceinline__ __nv_bfloat16 one(float v) { return __float2bfloat16_rn(v); }
    static __device__ __forceinline__ float to_float(__nv_bfloat16 v) { return __bfloat162float(v); }
    static constexpr double kMax = 3.3895313892515355e38;
};

// ---------------------------------------------------------------------------
// Prep kernels
// ---------------------------------------------------------------------------
// The mean of the centers per feature: a CTA per 32 features, lanes over
// features (coalesced rows), its 32 warps over the centers with four
// independent sums each (four loads in flight), the partial sums added in a
// fixed order (the same shift for the same centers).  Any shift keeps the
// labels exact: the bounds use the measured norms of the shifted, rounded
// operands.
constexpr int kShiftWarps = 32;
__global__ void __launch_bounds__(kShiftWarps * 32) shift_mean_kernel(const float *__restrict__ C, int d, int k,
                                                                      float *__restrict__ shift) {
    __shared__ double part[kShiftWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int f = blockIdx.x * 32 + lane;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    if (f < d) {
        const float *c = C + f;
        int j = w;
        for (; j + 3 * kShiftWarps < k; j += 4 * kShiftWarps) {
            const float a0 = __ldg(c + (int64_t)j * d);
            const float a1 = __ldg(c + (int64_t)(j + kShiftWarps) * d);
            const float a2 = __ldg(c + (int64_t)(j + 2 * kShiftWarps) * d);
            const float a3 = __ldg(c + (int64_t)(j + 3 * kShiftWarps) * d);
            s0 += (double)a0;
            s1 += (double)a1;
            s2 += (double)a2;
            s3 += (double)a3;
        }
        for (; j < k; j += kShiftWarps) s0 += (double)__ldg(c + (int64_t)j * d);
    }
    part[w][lane] = (s0 + s1) + (s2 + s3);
    __syncthreads();
    if (w == 0 && f < d) {
        double t = 0.0;
#pragma unroll 8
        for (int q = 0; q < kShiftWarps; ++q) t += part[q][lane];
        shift[f] = (float)(t / k);
    }
}

// Warp sum of per-lane compensated sums (s + c) in float32 (double-float
// style: TwoSum of the leading parts, errors carried in c): no float64 work,
// which is slow on this part.  Relative error a few units of float32.
__device__ __forceinline__ float warp_sum_ff(float s, float c) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float s2 = __shfl_xor_sync(0xffffffffu, s, off);
        const float c2 = __shfl_xor_sync(0xffffffffu, c, off);
        const float t = __fadd_rn(s, s2);
        const float bp = __fsub_rn(t, s);
        const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(s2, bp));
        s = t;
        c = __fadd_rn(__fadd_rn(c, c2), e);
    }
    return __fadd_rn(s, c);
}

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// ||c_j - m|| of every center (one warp each) and their maximum: picks the scale.
__global__ void center_norm_max_kernel(const float *__restrict__ C, int k, int d,
                                       const float *__restrict__ shift, uint32_t *__restrict__ scal) {
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (int64_t j = w; j < k; j += nw) {
        CSum s2;
        for (int f = lane; f < d; f += 32) {
            const float a = __fsub_rn(C[j * d + f], shift[f]);
            s2.add(a * a);
        }
        const double tot = warp_sum_d(s2.value());
        if (lane == 0) {
            const float nrm = (float)sqrt(tot);
            atomicMax(&scal[kScaleMax], nrm == nrm ? __float_as_uint(nrm) : 0x7f800000u);
        }
    }
}

// s = 2^sigma with s max||c'|| in (2^6, 2^7]; 1 when the centers coincide.
__global__ void scale_finalize_kernel(uint32_t *__restrict__ scal) {
    const float m = __uint_as_float(scal[kScaleMax]);
    int sigma = 0;
    if (m > 0.0f && m < __int_as_float(0x7f800000)) {
        int e;
        frexpf(m, &e);  // m = f 2^e, f in [0.5, 1): 2^(e-1) <= m < 2^e
        sigma = 7 - e;
        if (sigma > 60) sigma = 60;
        if (sigma < -60) sigma = -60;
    }
    scal[kScale] = __float_as_uint(ldexpf(1.0f, sigma));
    scal[kInvScale2] = __float_as_uint(ldexpf(1.0f, -2 * sigma));
}

// Frames: one warp per row.  xnorm = (||x_hat||^2 in scaled units, upper
// bound of ||x'||, upper bound of ||x_hat/s - x'||, 0) in unscaled units.
// get(f) gives feature f of row i.
template <typename T, class Get>
__device__ __forceinline__ void prep_one_row(const Get &get, int64_t i, int d, int kp,
                                             const float *__restrict__ shift, float sc, float inv_sc,
                                             T *__restrict__ xh, float4 *__restrict__ xnorm, float norm_inflate,
                                             int lane) {
    using O = Op16<T>;
    typename O::T2 *dst = reinterpret_cast<typename O::T2 *>(xh + i * kp);
    CSum h2, s2, e2;
    for (int f = 2 * lane; f < kp; f += 64) {
        // Columns < d: centered, scaled frame values; d and d+1: 1 (they
        // meet the hi/lo norm columns of the centers); the rest: 0.
        float a = 0.0f, b = 0.0f, ia, ib;
        if (f < d) {
            a = __fsub_rn(get(f), shift[f]);
            ia = a * sc;
        } else {
            ia = (f == d || f == d + 1) ? 1.0f : 0.0f;
        }
        if (f + 1 < d) {
            b = __fsub_rn(get(f + 1), shift[f + 1]);
            ib = b * sc;
        } else {
            ib = (f + 1 == d || f + 1 == d + 1) ? 1.0f : 0.0f;
        }
        const typename O::T2 h = O::pack(ia, ib);
        dst[f >> 1] = h;
        if (f < d) {
            const float ha = O::lo(h);
            const float ea = ha - ia;
            h2.add(ha * ha);
            s2.add(a * a);
            e2.add(ea * ea);
        }
        if (f + 1 < d) {
            const float hb = O::hi(h);
            const float eb = hb - ib;
            h2.add(hb * hb);
            s2.add(b * b);
            e2.add(eb * eb);
        }
    }
    const float th = warp_sum_ff(h2.s, h2.c);
    const float ts = warp_sum_ff(s2.s, s2.c);
    const float te = warp_sum_ff(e2.s, e2.c);
    if (lane == 0) {
        const float sx = __fsqrt_ru(__fmul_ru(ts, norm_inflate));
        const float hx = __fmul_ru(__fadd_ru(__fsqrt_ru(__fmul_ru(te, norm_inflate)), 1e-30f), inv_sc);
        xnorm[i] = make_float4(th, sx, hx, 0.0f);
    }
}

template <typename T, class Src>
__global__ void prep_frames_kernel(const Src rows, int64_t n, int d, int kp,
                                   const float *__restrict__ shift, const uint32_t *__restrict__ scal,
                                   T *__restrict__ xh, float4 *__restrict__ xnorm, float norm_inflate) {
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    const float sc = __uint_as_float(scal[kScale]);
    const float inv_sc = 1.0f / sc;  // exact: a power of two
    for (int64_t i = w; i < n; i += nw)
        prep_one_row<T>([&](int f) { return rows.get(i, f); }, i, d, kp, shift, sc, inv_sc, xh, xnorm,
                        norm_inflate, lane);
}

// The same for coordinate frames, with each frame's coordinates staged in
// one of two per-warp shared-memory slots by 4-byte cp.async copies (the
// next frame lands while this one is converted) and the atom pairs of all
// features in a CTA table of packed slot offsets (3 a | 3 b << 16).  The
// features are pair_feature's, as in PairRows.
constexpr int kPrepPairThreads = 256;
constexpr int kPrepPairMaxAtoms = 128;

size_t prep_pairs_smem(int d, int n_atoms) {
    const size_t slot = (size_t)((3 * n_atoms + 3) & ~3);
    return (size_t)((d + 3) & ~3) * 4 + (size_t)(kPrepPairThreads / 32) * 2 * slot * 4;
}

template <typename T>
__global__ void __launch_bounds__(kPrepPairThreads) prep_frames_pairs_kernel(
    const PairRows rows, int64_t n, int d, int kp, const float *__restrict__ shift,
    const uint32_t *__restrict__ scal, T *__restrict__ xh, float4 *__restrict__ xnorm, float norm_inflate) {
    extern __shared__ uint32_t prep_sm[];
    uint32_t *ofs = prep_sm;
    const int row_floats = 3 * rows.n_atoms;
    const int slot = (row_floats + 3) & ~3;
    const int lane = threadIdx.x & 31;
    float *ring = reinterpret_cast<float *>(prep_sm + ((d + 3) & ~3)) + (threadIdx.x >> 5) * 2 * slot;
    for (int f = threadIdx.x; f < d; f += blockDim.x) {
        const int2 pr = __ldg(rows.pairs + f);
        ofs[f] = (uint32_t)(3 * pr.x) | ((uint32_t)(3 * pr.y) << 16);
    }
    __syncthreads();
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float sc = __uint_as_float(scal[kScale]);
    const float inv_sc = 1.0f / sc;  // exact: a power of two
    auto fetch = [&](int64_t i, int q) {
        const float *g = rows.xyz + i * row_floats;
        float *dst = ring + q * slot;
        for (int t = lane; t < row_floats; t += 32) cp_async4(dst + t, g + t);
    };
    if (w < n) fetch(w, 0);
    cp_async_commit();
    int q = 0;
    for (int64_t i = w; i < n; i += nw, q ^= 1) {
        // the next frame into the other slot, read by every lane before the
        // __syncwarp that closed the previous row
        if (i + nw < n) fetch(i + nw, q ^ 1);
        cp_async_commit();
        cp_async_wait<1>();
        __syncwarp();
        const float *xr = ring + q * slot;
        prep_one_row<T>(
            [&](int f) {
                const uint32_t o = ofs[f];
                const float *a = xr + (o & 0xFFFFu);
                const float *b = xr + (o >> 16);
                return pair_feature(a[0], a[1], a[2], b[0], b[1], b[2]);
            },
            i, d, kp, shift, sc, inv_sc, xh, xnorm, norm_inflate, lane);
        __syncwarp();
    }
    cp_async_wait<0>();
}

// The same conversion with 16-byte loads (d % 4 == 0, 16-byte aligned X and
// shift): each lane owns 4 consecutive columns of every 128-column slice, and
// all of a row's loads are issued before any of its arithmetic, so a warp
// keeps the whole row in flight instead of one slice at a time.
template <typename T, int IT>  // 128-column slices per row: IT * 128 >= kp
__global__ void __launch_bounds__(256, 2) prep_frames_v4_kernel(const float *__restrict__ X, int64_t n, int d,
                                                                int kp, const float *__restrict__ shift,
                                                                const uint32_t *__restrict__ scal,
                                                                T *__restrict__ xh, float4 *__restrict__ xnorm,
                                                                float norm_inflate) {
    using O = Op16<T>;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    const float sc = __uint_as_float(scal[kScale]);
    const float inv_sc = 1.0f / sc;  // exact: a power of two
    auto load_row = [&](int64_t i, float4 (&v)[IT]) {
        const float *src = X + i * d;
#pragma unroll
        for (int it = 0; it < IT; ++it) {
            const int f = 4 * lane + 128 * it;
            v[it] = (i < n && f < d) ? __ldg(reinterpret_cast<const float4 *>(src + f)) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };
    float4 xv[IT];
    load_row(w, xv);
    for (int64_t i = w; i < n; i += nw) {
        // The next row's loads are in flight while this row is converted.
        float4 nx[IT];
        load_row(i + nw, nx);
        // ||x_hat||^2 enters the distance itself: a Kahan sum per lane (within
        // about 2u of the lane's terms; the distance bound allows 8u for this
        // norm).  The other two are bounds inflated by norm_inflate (far above
        // the few units of rounding of a plain per-lane sum): plain float32.
        float hs = 0.0f, hc = 0.0f;
        float s2 = 0.0f, e2 = 0.0f;
#pragma unroll
        for (int it = 0; it < IT; ++it) {
            const int f = 4 * lane + 128 * it;
            if (f >= kp) continue;
            const float4 s4 = f < d ? __ldg(reinterpret_cast<const float4 *>(shift + f)) : make_float4(0.f, 0.f, 0.f, 0.f);
            const float xa[4] = {xv[it].x, xv[it].y, xv[it].z, xv[it].w};
            const float sa[4] = {s4.x, s4.y, s4.z, s4.w};
            float a[4], ia[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                // Columns < d: centered, scaled frame values; d and d+1: 1
                // (they meet the hi/lo norm columns of the centers); the rest: 0.
                const int c = f + e;
                a[e] = c < d ? __fsub_rn(xa[e], sa[e]) : 0.0f;
                ia[e] = c < d ? a[e] * sc : ((c == d || c == d + 1) ? 1.0f : 0.0f);
            }
            const typename O::T2 h01 = O::pack(ia[0], ia[1]);
            const typename O::T2 h23 = O::pack(ia[2], ia[3]);
            uint2 packed;
            packed.x = *reinterpret_cast<const uint32_t *>(&h01);
            packed.y = *reinterpret_cast<const uint32_t *>(&h23);
            *reinterpret_cast<uint2 *>(xh + i * kp + f) = packed;
            const float hv[4] = {O::lo(h01), O::hi(h01), O::lo(h23), O::hi(h23)};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                if (f + e < d) {
                    const float ee = hv[e] - ia[e];
                    const float y = __fsub_rn(__fmul_rn(hv[e], hv[e]), hc);
                    const float t = __fadd_rn(hs, y);
                    hc = __fsub_rn(__fsub_rn(t, hs), y);
                    hs = t;
                    s2 = __fmaf_rn(a[e], a[e], s2);
                    e2 = __fmaf_rn(ee, ee, e2);
                }
            }
        }
        const float th = warp_sum_ff(hs, -hc);
        const float ts = warp_sum_ff(s2, 0.0f);
        const float te = warp_sum_ff(e2, 0.0f);
        if (lane == 0) {
            const float sx = __fsqrt_ru(__fmul_ru(ts, norm_inflate));
            const float hx = __fmul_ru(__fadd_ru(__fsqrt_ru(__fmul_ru(te, norm_inflate)), 1e-30f), inv_sc);
            xnorm[i] = make_float4(th, sx, hx, 0.0f);
        }
#pragma unroll
        for (int it = 0; it < IT; ++it) xv[it] = nx[it];
    }
}

// Centers: one warp per row of the k_pad-row block.  Columns d, d+1 hold the
// hi/lo FP16 split of -||c_hat||^2/2; cnorm = (upper bound of ||c'||, upper
// bound of ||c_hat/s - c'||).  A norm that FP16 cannot encode poisons cmax
// (every frame then takes the exact path).
template <typename T>
__global__ void prep_centers_kernel(const float *__restrict__ C, int k, int k_pad, int d, int kp,
                                    const float *__restrict__ shift, uint32_t *__restrict__ scal,
                                    T *__restrict__ ch, float2 *__restrict__ cnorm, float norm_inflate) {
    using O = Op16<T>;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    const float sc = __uint_as_float(scal[kScale]);
    const float inv_sc = 1.0f / sc;
    for (int64_t j = w; j < k; j += nw) {
        const float *src = C + j * d;
        typename O::T2 *dst = reinterpret_cast<typename O::T2 *>(ch + j * kp);
        double h2 = 0.0;
        CSum s2, e2;
        for (int f = 2 * lane; f < d; f += 64) {
            const float a = __fsub_rn(src[f], shift[f]);
            const float b = f + 1 < d ? __fsub_rn(src[f + 1], shift[f + 1]) : 0.0f;
            const typename O::T2 h = O::pack(a * sc, b * sc);
            const float ha = O::lo(h), hb = O::hi(h);
            h2 += (double)ha * ha + (double)hb * hb;
            s2.add(a * a);
            const float ea = ha - a * sc;
            e2.add(ea * ea);
            if (f + 1 < d) {
                s2.add(b * b);
                const float eb = hb - b * sc;
                e2.add(eb * eb);
            }
            dst[f >> 1] = h;
        }
        const double tot = warp_sum_d(h2);
        const double ts = warp_sum_d(s2.value());
        const double te = warp_sum_d(e2.value());
        __syncwarp();  // the pair writes above land before lane 0 writes columns d, d+1
        if (lane == 0) {
            const double val = -0.5 * tot;
            const T hi = O::one((float)val);
            const T lo = O::one((float)(val - (double)O::to_float(hi)));
            T *row = ch + j * kp;
            row[d] = hi;
            row[d + 1] = lo;
            const float nrm = __fsqrt_ru(__fmul_ru((float)ts, norm_inflate));
            const float hc = __fmul_ru(__fadd_ru(__fsqrt_ru(__fmul_ru((float)te, norm_inflate)), 1e-30f), inv_sc);
            cnorm[j] = make_float2(nrm, hc);
            const bool encodable = fabs(val) < O::kMax && nrm == nrm && hc == hc;
            atomicMax(&scal[kCmax], encodable ? __float_as_uint(nrm) : 0x7f800000u);
            atomicMax(&scal[kHcMax], encodable ? __float_as_uint(hc) : 0x7f800000u);
        }
    }
    for (int64_t j = k + w; j < k_pad; j += nw)
        if (lane == 0) cnorm[j] = make_float2(0.0f, 0.0f);
}

// ---------------------------------------------------------------------------
// FP8 (e4m3) operands.  e4m3 has 3 mantissa bits and spans 2^-9 .. 448, too
// narrow to carry the center norms in extra GEMM columns, so the epilogue
// adds -||c~_j||^2 / 2 itself.  A frame row may take its own power-of-two
// scale s_i (a row's scale does not change its argmin): max |x'| s_i lies in
// [128, 256).  The centers share one scale t with max |c'| t in [128, 256).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint8_t to_e4m3(float v) {
    return (uint8_t)__nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3);
}

__device__ __forceinline__ float from_e4m3(uint8_t q) {
    const __half_raw h = __nv_cvt_fp8_to_halfraw((__nv_fp8_storage_t)q, __NV_E4M3);
    return __half2float(__half(h));
}

// The power of two s with m s in [128, 256) (m > 0 finite), else 0.
__device__ __forceinline__ float fp8_scale_for(float m) {
    if (!(m > 0.0f) || !(m <= 3.4028234663852886e38f)) return 0.0f;
    int e;
    frexpf(m, &e);  // 2^(e-1) <= m < 2^e
    const int sigma = 8 - e;
    if (sigma > 126 || sigma < -126) return 0.0f;
    return ldexpf(1.0f, sigma);
}

// max |c'_jf| over all centers (float bits; a NaN poisons it to +inf).
__global__ void center_absmax_kernel(const float *__restrict__ C, int k, int d, const float *__restrict__ shift,
                                     uint32_t *__restrict__ scal) {
    float m = 0.0f;
    const int64_t total = (int64_t)k * d;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const float a = fabsf(__fsub_rn(C[e], shift[e % d]));
        m = a == a ? fmaxf(m, a) : __int_as_float(0x7f800000);
    }
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(&scal[kScaleMax], __float_as_uint(m));
}

// t for the FP8 centers (1 when they coincide or are not finite).
__global__ void scale_fp8_finalize_kernel(uint32_t *__restrict__ scal) {
    const float t = fp8_scale_for(__uint_as_float(scal[kScaleMax]));
    scal[kScale] = __float_as_uint(t > 0.0f ? t : 1.0f);
    scal[kInvScale2] = __float_as_uint(1.0f);
}

// Frames: one warp per row.  xnorm = (||x~||^2, upper bound of ||x'||, upper
// bound of ||x~ - x'||, 1 / (s_i t)), x~ = e4m3(x' s_i) / s_i, in unscaled
// units.  A row without a usable scale (all zero: s_i = 1; non-finite:
// infinite bounds, which send it to the exact pass) is still written.
__global__ void prep_frames_fp8_kernel(const float *__restrict__ X, int64_t n, int d, int kp,
                                       const float *__restrict__ shift, const uint32_t *__restrict__ scal,
                                       uint8_t *__restrict__ xq, float4 *__restrict__ xnorm, float norm_inflate) {
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    const float t = __uint_as_float(scal[kScale]);
    for (int64_t i = w; i < n; i += nw) {
        const float *src = X + i * d;
        float m = 0.0f;
        bool bad = false;
        for (int f = lane; f < d; f += 32) {
            const float a = fabsf(__fsub_rn(src[f], shift[f]));
            bad |= !(a <= 3.4028234663852886e38f);
            m = fmaxf(m, a);
        }
        for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
        bad = __any_sync(0xffffffffu, bad);
        float si = fp8_scale_for(m);
        if (si == 0.0f) {
            bad |= m != 0.0f;
            si = 1.0f;
        }
        const float inv_si = 1.0f / si;  // exact: a power of two
        float hs = 0.0f, hc = 0.0f, s2 = 0.0f, e2 = 0.0f;
        uint32_t *dst = reinterpret_cast<uint32_t *>(xq + i * kp);
        for (int f = 4 * lane; f < kp; f += 128) {
            uint32_t word = 0u;
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int c = f + e;
                if (c < d) {
                    const float a = __fsub_rn(src[c], shift[c]);
                    const float as = a * si;
                    const uint8_t q = to_e4m3(as);
                    const float qv = from_e4m3(q);
                    word |= (uint32_t)q << (8 * e);
                    const float xt = qv * inv_si;  // exact
                    const float y = __fsub_rn(__fmul_rn(xt, xt), hc);
                    const float tt = __fadd_rn(hs, y);
                    hc = __fsub_rn(__fsub_rn(tt, hs), y);
                    hs = tt;
                    s2 = __fmaf_rn(a, a, s2);
                    const float ee = qv - as;
                    e2 = __fmaf_rn(ee, ee, e2);
                }
            }
            dst[f >> 2] = word;
        }
        const float th = warp_sum_ff(hs, -hc);
        const float ts = warp_sum_ff(s2, 0.0f);
        const float te = warp_sum_ff(e2, 0.0f);
        if (lane == 0) {
            const float inf = __int_as_float(0x7f800000);
            const float inv_st = 1.0f / (si * t);  // exact while si t is a normal float
            bad |= !(inv_st >= 1.1754943508222875e-38f && inv_st <= 3.4028234663852886e38f);
            const float sx = bad ? inf : __fsqrt_ru(__fmul_ru(ts, norm_inflate));
            const float hx = bad ? inf : __fmul_ru(__fadd_ru(__fsqrt_ru(__fmul_ru(te, norm_inflate)), 1e-30f), inv_si);
            xnorm[i] = make_float4(bad ? 0.0f : th, sx, hx, bad ? 1.0f : inv_st);
        }
    }
}

// Centers: one warp per row of the k_pad-row block.  cnorm = (upper bound of
// ||c'||, upper bound of ||c~ - c'||), chn = -||c~||^2 / 2 (in double, then
// rounded), c~ = e4m3(c' t) / t.  A center that e4m3 cannot represent
// poisons cmax (every frame then takes the exact path).
__global__ void prep_centers_fp8_kernel(const float *__restrict__ C, int k, int k_pad, int d, int kp,
                                        const float *__restrict__ shift, uint32_t *__restrict__ scal,
                                        uint8_t *__restrict__ cq, float2 *__restrict__ cnorm, float *__restrict__ chn,
                                        float norm_inflate) {
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    const float t = __uint_as_float(scal[kScale]);
    const float inv_t = 1.0f / t;
    for (int64_t j = w; j < k; j += nw) {
        const float *src = C + j * d;
        uint32_t *dst = reinterpret_cast<uint32_t *>(cq + j * kp);
        double h2 = 0.0;
        CSum s2, e2;
        for (int f = 4 * lane; f < kp; f += 128) {
            uint32_t word = 0u;
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int c = f + e;
                if (c < d) {
                    const float a = __fsub_rn(src[c], shift[c]);
                    const float at = a * t;
                    const uint8_t q = to_e4m3(at);
                    const float qv = from_e4m3(q);
                    word |= (uint32_t)q << (8 * e);
                    const double ct = (double)qv * (double)inv_t;
                    h2 += ct * ct;
                    s2.add(a * a);
                    const float ee = qv - at;
                    e2.add(ee * ee);
                }
            }
            dst[f >> 2] = word;
        }
        const double tot = warp_sum_d(h2);
        const double ts = warp_sum_d(s2.value());
        const double te = warp_sum_d(e2.value());
        if (lane == 0) {
            const float nrm = __fsqrt_ru(__fmul_ru((float)ts, norm_inflate));
            const float hc = __fmul_ru(__fadd_ru(__fsqrt_ru(__fmul_ru((float)te, norm_inflate)), 1e-30f), inv_t);
            cnorm[j] = make_float2(nrm, hc);
            const float hn = (float)(-0.5 * tot);
            chn[j] = hn;
            const bool ok = hn == hn && fabsf(hn) <= 3.4028234663852886e38f && nrm == nrm && hc == hc;
            atomicMax(&scal[kCmax], ok ? __float_as_uint(nrm) : 0x7f800000u);
            atomicMax(&scal[kHcMax], ok ? __float_as_uint(hc) : 0x7f800000u);
        }
    }
    for (int64_t j = k + w; j < k_pad; j += nw)
        if (lane == 0) {
            cnorm[j] = make_float2(0.0f, 0.0f);
            chn[j] = 0.0f;
        }
}

// ---------------------------------------------------------------------------
// Main kernel
// ---------------------------------------------------------------------------
// A lower bound of the tensor-core accumulator of frame row xr and center
// row cr (kp 16-bit operands each, 16-byte aligned rows): the float32 dot
// product F of the two rows (every product exact, one rounding per fused
// multiply-add, so within seed_coef S of the exact sum, S = sum |a b|),
// less seed_coef S and less tc_err, the accumulation allowance of the MMA.
template <typename T>
__device__ __forceinline__ float accumulator_floor(const T *__restrict__ xr, const T *__restrict__ cr, int kp,
                                                   float seed_coef, float tc_err) {
    using O = Op16<T>;
    const uint4 *x4 = reinterpret_cast<const uint4 *>(xr);
    const uint4 *c4 = reinterpret_cast<const uint4 *>(cr);
    float F = 0.0f, S = 0.0f;
    for (int q = 0; q < kp / 8; ++q) {
        const uint4 xa = __ldg(x4 + q), ca = __ldg(c4 + q);
        const uint32_t xw[4] = {xa.x, xa.y, xa.z, xa.w}, cw[4] = {ca.x, ca.y, ca.z, ca.w};
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            typename O::T2 xp, cp;
            memcpy(&xp, &xw[h], 4);
            memcpy(&cp, &cw[h], 4);
            const float a0 = O::lo(xp), a1 = O::hi(xp), b0 = O::lo(cp), b1 = O::hi(cp);
            F = fmaf(a0, b0, F);
            F = fmaf(a1, b1, F);
            S = __fadd_ru(S, fabsf(a0 * b0));
            S = __fadd_ru(S, fabsf(a1 * b1));
        }
    }
    // 1e-30 covers products below float32's normal range (BF16 operands)
    return __fsub_rd(__fsub_rd(F, __fmul_ru(seed_coef, S)), tc_err) - 1e-30f;
}

__device__ __forceinline__ float lo_bound(float v, float E, float R, float g_lo) {
    float a = __fsqrt_rd(fmaxf(__fsub_rd(v, E), 0.0f));
    a = fmaxf(__fsub_rd(a, R), 0.0f);
    return __fmul_rd(__fmul_rd(a, a), g_lo) - 1e-37f;
}

__device__ __forceinline__ float hi_bound(float v, float E, float R, float g_hi) {
    float a = __fadd_ru(__fsqrt_ru(fmaxf(__fadd_ru(v, E), 0.0f)), R);
    return __fadd_ru(__fmul_ru(__fmul_ru(a, a), g_hi), 1e-37f);
}

// Rounding of the float32 centering x' = fl(x - m): at most 2^-24 |x - m|
// per component, so 2^-23 (sx + sc) covers both operands.
constexpr float kCenterEps = 1.1920929e-07f;  // 2^-23

// Smallest accumulator a' that can still belong to a possible argmin, given
// the best accumulator so far: with H = (sqrt(vb + E) + R)^2 g_hi the upper
// end of the best distance, lo(v') <= H needs v' <= V = (sqrt(H / g_lo) + R)^2
// + E (worst-case R, E), and v' = (||x_hat||^2 - 2 a') / s^2.  The root of
// H / g_lo is (sqrt(vb + E) + R) sqrt(g_hi / g_lo): g_ratio is that factor
// inflated by 2^-19 (more than the roundings of the literal form), and
// R_pad = R + 1e-18 covers the root of hi_bound's 1e-37 term.  Rounded
// towards admitting more throughout; one root, no division.
__device__ __forceinline__ float window_threshold(float best, float xn2, float inv_s2, float s2, float E,
                                                  float R, float R_pad, float g_ratio) {
    const float vb = fmaf(-2.0f, best, xn2) * inv_s2;
    const float a = __fadd_ru(__fsqrt_ru(fmaxf(__fadd_ru(vb, E), 0.0f)), R);
    const float q = __fadd_ru(__fmul_ru(g_ratio, a), R_pad);
    const float V = __fadd_ru(__fmul_ru(q, q), E);
    const float t = __fmul_rd(__fsub_rd(xn2, __fmul_ru(V, s2)), 0.5f);
    return __fsub_rd(t, __fmul_ru(fabsf(t), 1e-6f)) - 1e-30f;
}

// PAIR: a cluster of two CTAs on two SMs computes M = 256 tiles with
// tcgen05 cta_group::2.  Each CTA keeps its own 128 frames (A) resident and
// loads half of every 256-center B stage; the leader CTA (rank 0) issues the
// MMAs, which read A and B from both CTAs' shared memory and write each CTA's
// own accumulator rows.  All barriers the MMAs wait on live in the leader
// (the peer's copies and accumulator releases arrive there); the MMA commits
// arrive in both CTAs.
// L: candidates kept per frame (a register list; 8 or 16).  F8: e4m3
// operands (128 elements per 128-byte chunk, kind::f8f6f4); the epilogue
// turns the accumulator into a_j = acc_j / (s_i t) - ||c~_j||^2 / 2 with the
// frame's scale s_i and the centers' t, in unscaled units.
template <bool PAIR, int L, bool F8>
__global__ void __launch_bounds__(kThreadsTC, 1)
    tc_assign_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                     const TcParams p) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    // Resident mode: sA holds the frame tile's nkc A chunks, the ring of
    // stages holds B.  Streaming mode (d too large for a resident tile):
    // every stage holds one A chunk followed by the matching B chunk.
    const bool stream = p.stream_a != 0;
    const int nab = stream ? 0 : p.nkc;  // resident A chunks (and their barrier pairs)
    uint8_t *sA = smem;
    uint8_t *sB = sA + nab * kABytesPerChunk;
    const int b_stage_bytes = (PAIR ? p.bn / 2 : p.bn) * kKC * 2;
    const int stage_bytes = b_stage_bytes + (stream ? kABytesPerChunk : 0);
    const int b_off = stream ? kABytesPerChunk : 0;  // B within a stage
    uint64_t *bars = reinterpret_cast<uint64_t *>(sB + p.stages * stage_bytes);
    uint64_t *a_full = bars;
    uint64_t *a_empty = a_full + nab;
    uint64_t *b_full = a_empty + nab;
    uint64_t *b_empty = b_full + p.stages;
    uint64_t *acc_full = b_empty + p.stages;
    uint64_t *acc_empty = acc_full + 2;
    uint64_t *drain = acc_empty + 2;
    uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(drain + 1);
    volatile uint32_t *abort_flag = tmem_holder + 1;

    constexpr int KC = F8 ? 128 : kKC;  // elements per 128-byte chunk
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t rank = PAIR ? cluster_ctarank() : 0u;
    const bool leader = rank == 0;
    // Frame units: 128 frames per CTA; a pair takes 256 consecutive frames,
    // its rank-r CTA the r-th half.
    const int64_t unit = PAIR ? 2 * kBM : kBM;
    const int64_t n_units = (p.n - p.frame0 + unit - 1) / unit;
    const int64_t unit0 = PAIR ? blockIdx.x / 2 : blockIdx.x;
    const int64_t unit_stride = PAIR ? gridDim.x / 2 : gridDim.x;

    if (threadIdx.x == 0) {
        for (int c = 0; c < nab; ++c) {
            mbar_init(&a_full[c], 1);
            mbar_init(&a_empty[c], 1);
        }
        for (int s = 0; s < p.stages; ++s) {
            mbar_init(&b_full[s], 1);
            mbar_init(&b_empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], PAIR ? 8 : 4);  // the epilogue warps of one or both CTAs
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == 1) {
        if (PAIR) {  // one warp of each CTA of the pair
            tmem_alloc_pair(tmem_holder, p.tmem_cols);
            tmem_relinquish_pair();
        } else {
            tmem_alloc(tmem_holder, p.tmem_cols);
            tmem_relinquish();
        }
    }
    tc_fence_before();
    __syncthreads();
    if (PAIR) cluster_sync_all();  // both CTAs' barriers are initialised before any remote arrive
    tc_fence_after();
    const uint32_t tmem_base = *tmem_holder;

    if (warp == 0) {
        // ---------------- TMA producer ----------------
        // The whole warp runs the loop (waits by all lanes, agreed by vote);
        // one elected lane issues the copies.  Per center tile: B stages
        // t = 0..nbst-1 of 64 K-columns each; in the resident form the A
        // chunk t (the same 64 columns) is loaded with stage t of the first
        // center tile, in the streaming form it travels inside every stage.
        // Stage index and phase advance incrementally; a failed wait clears
        // ok and stops the issues, and the warp agrees on ok once per center
        // tile.  `issued` counts the B stages actually loaded (for the drain).
        uint32_t issued = 0, a_issued_tiles = 0;
        uint32_t t_local = 0;
        bool ok = true;
        unsigned long long w_b = 0, w_a = 0;
        unsigned long long *pw_b = (p.wait_cycles && lane == 0) ? &w_b : nullptr;
        unsigned long long *pw_a = (p.wait_cycles && lane == 0) ? &w_a : nullptr;
        uint32_t s = 0, sph = 0;
        for (int64_t ft = unit0; ft < n_units && ok; ft += unit_stride, ++t_local) {
            const int frame_row = (int)(p.frame0 + ft * unit + rank * kBM);
            for (int ct = 0; ct < p.n_ctiles && ok; ++ct) {
                for (int t = 0; t < p.nbst; ++t) {
                    if (!stream && ct == 0) {
                        if (ok) ok = mbar_wait_timed(&a_empty[t], (t_local & 1u) ^ 1u, pw_a);
                        if (elect_one() && ok) {
                            if (PAIR) {
                                if (leader) mbar_arrive_expect_tx(&a_full[t], 2 * kABytesPerChunk);
                                tma_load_2d_pair(sA + t * kABytesPerChunk, &tmA, t * KC, frame_row,
                                                 mapa_shared(smem_u32(&a_full[t]), 0));
                            } else {
                                mbar_arrive_expect_tx(&a_full[t], kABytesPerChunk);
                                tma_load_2d(sA + t * kABytesPerChunk, &tmA, t * KC, frame_row, &a_full[t]);
                            }
                        }
                        __syncwarp();
                    }
                    if (ok) ok = mbar_wait_timed(&b_empty[s], sph ^ 1u, pw_b);
                    if (elect_one() && ok) {
                        uint8_t *st = sB + s * stage_bytes;
                        if (PAIR) {
                            if (leader) mbar_arrive_expect_tx(&b_full[s], 2 * stage_bytes);
                            tma_load_2d_pair(st, &tmB, t * KC, ct * p.bn + (int)rank * (p.bn / 2),
                                             mapa_shared(smem_u32(&b_full[s]), 0));
                        } else {
                            mbar_arrive_expect_tx(&b_full[s], stage_bytes);
                            if (stream) tma_load_2d(st, &tmA, t * KC, frame_row, &b_full[s]);
                            tma_load_2d(st + b_off, &tmB, t * KC, ct * p.bn, &b_full[s]);
                        }
                        ++issued;
                    }
                    __syncwarp();
                    if (++s == (uint32_t)p.stages) {
                        s = 0;
                        sph ^= 1u;
                    }
                }
                if (ct == 0) a_issued_tiles += 1;
                ok = __all_sync(0xffffffffu, ok) && !__any_sync(0xffffffffu, *abort_flag != 0);
            }
        }
        issued = __shfl_sync(0xffffffffu, issued, 0);  // lane 0 is the elected lane of a full warp
        if (!ok && lane == 0) {
            atomicOr(p.err, (uint32_t)kDevTimeoutTma);
            *abort_flag = 1;
        }
        if (pw_b) {
            atomicAdd(&p.wait_cycles[kWaitProdB], w_b);
            atomicAdd(&p.wait_cycles[kWaitProdA], w_a);
        }
        // Drain: every load issued above has landed before the CTA exits
        // (the A chunks of the last frame tile whose loads were issued, and
        // the last issued load of every B stage).  In a pair the barriers are
        // the leader's and count both CTAs' copies; the peer is held by the
        // closing cluster barrier until the leader has drained.
        if ((!PAIR || leader) && a_issued_tiles > 0) {
            const uint32_t last_a = (a_issued_tiles - 1u) & 1u;
            for (int kc = 0; kc < nab; ++kc) mbar_wait(&a_full[kc], last_a);
        }
        for (uint32_t st = 0; (!PAIR || leader) && st < (uint32_t)p.stages && st < issued; ++st) {
            const uint32_t last_q = issued - 1u - ((issued - 1u - st) % p.stages);
            mbar_wait(&b_full[st], (last_q / p.stages) & 1u);
        }
        __syncwarp();
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        // Converged warp; one elected lane issues the MMAs and commits.  The
        // shared-memory descriptors advance by adding to their start-address
        // field (addresses stay below 256 KB); a failed wait clears ok and
        // stops the issues (the elected lane, lane 0 of the converged warp,
        // decides by its own wait), and the warp agrees on ok once per
        // center tile.
        // In a pair only the leader issues; the peer's MMA warp waits for
        // the drain commit below.
        const uint32_t idesc = make_idesc(PAIR ? 2 * kBM : kBM, p.bn, p.bf16 != 0);
        const uint64_t adesc0 = sw128_desc(smem_u32(sA));
        const uint64_t sdesc0 = sw128_desc(smem_u32(sB));
        const uint64_t sstep = (uint64_t)(stage_bytes >> 4);
        const uint64_t boff = (uint64_t)(b_off >> 4);
        const uint64_t astep = (uint64_t)(kABytesPerChunk >> 4);
        const int last_steps = p.ksteps_total - 4 * (p.nbst - 1);  // 1..4
        uint32_t accq = 0, t_local = 0;
        bool ok = true;
        unsigned long long w_b = 0, w_a = 0, w_acc = 0;
        const long long t_start = clock64();
        const bool diag = p.wait_cycles && lane == 0 && (!PAIR || leader);
        unsigned long long *pw_b = diag ? &w_b : nullptr;
        unsigned long long *pw_a = diag ? &w_a : nullptr;
        unsigned long long *pw_acc = diag ? &w_acc : nullptr;
        uint32_t s = 0, sph = 0;  // B stage and its phase
        uint64_t sdesc = sdesc0;  // descriptor of stage s
        for (int64_t ft = unit0; (!PAIR || leader) && ft < n_units && ok; ft += unit_stride, ++t_local) {
            for (int ct = 0; ct < p.n_ctiles && ok; ++ct) {
                const uint32_t buf = accq & 1u;
                // The peer CTA's epilogue warps arrive here too (cluster scope).
                ok = PAIR ? mbar_wait_cluster_timed(&acc_empty[buf], ((accq >> 1) & 1u) ^ 1u, pw_acc)
                          : mbar_wait_timed(&acc_empty[buf], ((accq >> 1) & 1u) ^ 1u, pw_acc);
                tc_fence_after();
                const uint32_t d_tmem = tmem_base + buf * (uint32_t)p.bn;
                const bool first = ct == 0, last = ct == p.n_ctiles - 1;
                uint64_t ad = adesc0;
                for (int t = 0; t < p.nbst; ++t) {
                    if (!stream && first && ok) ok = mbar_wait_timed(&a_full[t], t_local & 1u, pw_a);
                    if (ok) ok = mbar_wait_timed(&b_full[s], sph, pw_b);
                    // TMA completion on the mbarrier orders the loaded tiles before
                    // the MMAs; no tcgen05 fence is needed here.
                    const uint64_t a_d = stream ? sdesc : ad;
                    const uint64_t b_d = sdesc + boff;
                    const int steps = t == p.nbst - 1 ? last_steps : 4;
                    if (elect_one() && ok) {
                        if (PAIR) {
                            mma_op_pair<F8>(d_tmem, a_d, b_d, idesc, t != 0);
#pragma unroll
                            for (int kk = 1; kk < 4; ++kk)
                                if (kk < steps) mma_op_pair<F8>(d_tmem, a_d + 2 * kk, b_d + 2 * kk, idesc, 1u);
                            mma_commit_pair(&b_empty[s]);
                            if (last) mma_commit_pair(&a_empty[t]);
                        } else {
                            mma_op<F8>(d_tmem, a_d, b_d, idesc, t != 0);
#pragma unroll
                            for (int kk = 1; kk < 4; ++kk)  // 32-byte K steps: +2 in the start-address field
                                if (kk < steps) mma_op<F8>(d_tmem, a_d + 2 * kk, b_d + 2 * kk, idesc, 1u);
                            mma_commit(&b_empty[s]);
                            if (!stream && last) mma_commit(&a_empty[t]);
                        }
                    }
                    __syncwarp();
                    ad += astep;
                    if (++s == (uint32_t)p.stages) {
                        s = 0;
                        sph ^= 1u;
                        sdesc = sdesc0;
                    } else {
                        sdesc += sstep;
                    }
                }
                ok = __all_sync(0xffffffffu, ok);
                if (!ok) break;
                if (elect_one()) {
                    if (PAIR)
                        mma_commit_pair(&acc_full[buf]);
                    else
                        mma_commit(&acc_full[buf]);
                }
                __syncwarp();
                ++accq;
                if (__any_sync(0xffffffffu, *abort_flag != 0)) ok = false;
            }
        }
        if (!ok && lane == 0) {
            atomicOr(p.err, (uint32_t)kDevTimeoutMma);
            *abort_flag = 1;
        }
        if (pw_b) {
            atomicAdd(&p.wait_cycles[kWaitMmaB], w_b);
            atomicAdd(&p.wait_cycles[kWaitMmaA], w_a);
            atomicAdd(&p.wait_cycles[kWaitMmaAcc], w_acc);
            atomicAdd(&p.wait_cycles[kMmaTotal], (unsigned long long)(clock64() - t_start));
        }
        // Drain: all issued MMAs complete before TMEM is released (in a pair
        // the leader's commit arrives on both CTAs' drain barriers).
        if (elect_one()) {
            if (!PAIR)
                mma_commit(drain);
            else if (leader)
                mma_commit_pair(drain);
        }
        __syncwarp();
        mbar_wait(drain, 0);
        __syncwarp();
    } else if (warp >= 2) {
        // ---------------- epilogue ----------------
        const int quarter = warp & 3;
        const int row = quarter * 32 + lane;
        const uint32_t lane_off = (uint32_t)(quarter * 32) << 16;
        // FP8 works in unscaled units (the epilogue divides by s_i t).
        const float inv_s2 = F8 ? 1.0f : __uint_as_float(p.scal[kInvScale2]);
        const float s2 = 1.0f / inv_s2;  // exact: a power of two
        const float sc_max = __uint_as_float(p.scal[kCmax]);
        const float hc_max = __uint_as_float(p.scal[kHcMax]);
        const float kNegInf = __int_as_float(0xff800000);
        const float kInf = __int_as_float(0x7f800000);
        uint32_t accq = 0;
        bool ok = true;
        unsigned long long w_acc = 0;
        const long long t_start = clock64();
        unsigned long long *pw_acc = (p.wait_cycles && warp == 2 && lane == 0) ? &w_acc : nullptr;
        for (int64_t ft = unit0; ft < n_units && ok; ft += unit_stride) {
            const int64_t i = p.frame0 + ft * unit + (int64_t)rank * kBM + row;
            const float4 xn = i < p.n ? p.xnorm[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            // Worst-case bound terms over all centers: the acceptance window
            // and the overflow decision use them.
            const float smax = xn.y + sc_max;
            const float Rmax = __fadd_ru(__fadd_ru(xn.z, hc_max), __fmul_ru(kCenterEps, smax));
            const float Emax = __fmul_ru(p.e_coef, __fmul_ru(smax, smax));
            const float Rpad = __fadd_ru(Rmax, 1e-18f);
            float best = kNegInf, thr = kNegInf;
            if (!F8 && p.seed_xh && i < p.n) {
                // Seed: a lower bound of the accumulator of the center the
                // frame's label names (the previous iteration's, where there
                // is one; any center in range is valid).  The true maximum is
                // at least as large, so the threshold only starts higher and
                // no candidate is lost; the frame's lists stay short.
                const int pl = p.labels[i];
                if (pl >= 0 && pl < p.k) {
                    const float2 cn = p.cnorm[pl];
                    const float sj = xn.y + cn.x;
                    const float Ej = __fmul_ru(p.e_coef, __fmul_ru(sj, sj));
                    const float tc_err = __fmul_ru(__fmul_ru(Ej, s2), 0.5f);
                    const size_t xo = (size_t)i * p.kp, co = (size_t)pl * p.kp;
                    const float seed =
                        p.bf16 ? accumulator_floor(static_cast<const __nv_bfloat16 *>(p.seed_xh) + xo,
                                                   static_cast<const __nv_bfloat16 *>(p.seed_ch) + co, p.kp,
                                                   p.seed_coef, tc_err)
                               : accumulator_floor(static_cast<const __half *>(p.seed_xh) + xo,
                                                   static_cast<const __half *>(p.seed_ch) + co, p.kp, p.seed_coef,
                                                   tc_err);
                    if (seed > kNegInf && seed < kInf) {
                        best = seed;
                        thr = window_threshold(best, xn.x, inv_s2, s2, Emax, Rmax, Rpad, p.g_ratio);
                    }
                }
            }
            bool ovf = false;
            float la[L];
            int lid[L];
#pragma unroll
            for (int m = 0; m < L; ++m) {
                la[m] = kNegInf;
                lid[m] = -1;
            }
            for (int ct = 0; ct < p.n_ctiles; ++ct) {
                const uint32_t buf = accq & 1u;
                const bool got = __all_sync(0xffffffffu, mbar_wait_timed(&acc_full[buf], (accq >> 1) & 1u, pw_acc));
                if (!got) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t tbase = tmem_base + lane_off + buf * (uint32_t)p.bn;
                for (int cc = 0; cc < p.bn; cc += 32) {
                    uint32_t r[32];
                    tmem_ld32(tbase + cc, r);
                    tmem_wait_ld();
                    const int j0 = ct * p.bn + cc;
                    float v[32];
                    if (F8) {
                        // a_j = acc_j / (s_i t) - ||c~_j||^2 / 2 (xn.w = 1 / (s_i t), a power of two)
                        const float4 *hn = reinterpret_cast<const float4 *>(p.chn + j0);
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            const float4 h = __ldg(hn + q);
                            v[4 * q + 0] = fmaf(__uint_as_float(r[4 * q + 0]), xn.w, h.x);
                            v[4 * q + 1] = fmaf(__uint_as_float(r[4 * q + 1]), xn.w, h.y);
                            v[4 * q + 2] = fmaf(__uint_as_float(r[4 * q + 2]), xn.w, h.z);
                            v[4 * q + 3] = fmaf(__uint_as_float(r[4 * q + 3]), xn.w, h.w);
                        }
                    } else {
#pragma unroll
                        for (int c = 0; c < 32; ++c) v[c] = __uint_as_float(r[c]);
                    }
                    if (j0 + 32 > p.k) {
#pragma unroll
                        for (int c = 0; c < 32; ++c)
                            if (j0 + c >= p.k) v[c] = kNegInf;
                    }
                    if (p.dump && i < p.n) {
#pragma unroll
                        for (int c = 0; c < 32; ++c)
                            if (j0 + c < p.k) p.dump[i * p.k + j0 + c] = fmaf(-2.0f, v[c], xn.x) * inv_s2;
                    }
                    // Chunk maximum by a tree of three-input maxima: 16
                    // instructions in four dependent steps (32 -> 12 -> 4 -> 2 -> 1).
                    float m12[12];
#pragma unroll
                    for (int q = 0; q < 10; ++q) m12[q] = max3f(v[3 * q], v[3 * q + 1], v[3 * q + 2]);
                    m12[10] = v[30];
                    m12[11] = v[31];
                    const float m4a = max3f(m12[0], m12[1], m12[2]);
                    const float m4b = max3f(m12[3], m12[4], m12[5]);
                    const float m4c = max3f(m12[6], m12[7], m12[8]);
                    const float m4d = max3f(m12[9], m12[10], m12[11]);
                    const float mx = fmaxf(max3f(m4a, m4b, m4c), m4d);
                    if (mx >= thr && mx > kNegInf) {
                        if (mx > best) {
                            best = mx;
                            thr = window_threshold(best, xn.x, inv_s2, s2, Emax, Rmax, Rpad, p.g_ratio);
                        }
                        // Columns at or above the threshold as a bit mask; each
                        // one is pushed on the list.  A lone column is the
                        // chunk's maximum; otherwise each value is picked out
                        // of the registers by a select tree over the bits of
                        // its index.
                        unsigned mk[4] = {0u, 0u, 0u, 0u};  // four independent chains
#pragma unroll
                        for (int c = 0; c < 32; ++c) mk[c & 3] |= (v[c] >= thr ? 1u : 0u) << c;
                        unsigned msk = (mk[0] | mk[1]) | (mk[2] | mk[3]);
                        const int nv = p.k - j0;
                        if (nv < 32) msk &= nv > 0 ? (1u << nv) - 1u : 0u;
                        const bool lone = (msk & (msk - 1u)) == 0u;
                        while (msk) {
                            const int c = __ffs(msk) - 1;
                            msk &= msk - 1u;
                            float vc = mx;
                            if (!lone) {
                                float t16[16], t8[8], t4[4], t2[2];
#pragma unroll
                                for (int q = 0; q < 16; ++q) t16[q] = (c & 16) ? v[q + 16] : v[q];
#pragma unroll
                                for (int q = 0; q < 8; ++q) t8[q] = (c & 8) ? t16[q + 8] : t16[q];
#pragma unroll
                                for (int q = 0; q < 4; ++q) t4[q] = (c & 4) ? t8[q + 4] : t8[q];
#pragma unroll
                                for (int q = 0; q < 2; ++q) t2[q] = (c & 2) ? t4[q + 2] : t4[q];
                                vc = (c & 1) ? t2[1] : t2[0];
                            }
                            if (lid[L - 1] >= 0 && la[L - 1] >= thr) ovf = true;
#pragma unroll
                            for (int m = L - 1; m > 0; --m) {
                                la[m] = la[m - 1];
                                lid[m] = lid[m - 1];
                            }
                            la[0] = vc;
                            lid[0] = j0 + c;
                        }
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) {
                    if (PAIR)
                        mbar_arrive_cluster(mapa_shared(smem_u32(&acc_empty[buf]), 0));
                    else
                        mbar_arrive(&acc_empty[buf]);
                }
                ++accq;
            }
            if (!ok) break;

            // ---- decision ----
            bool need_rc = false, need_full = false;
            unsigned cmask = 0;  // bit m: list entry m is a candidate
            int jb = 0;          // candidate with the largest accumulator
            float lo[L];        // lower bounds of the candidates' exact distances
            if (i < p.n) {
                float vv[L], RR[L], EE[L];
                float H = kInf;
#pragma unroll
                for (int m = 0; m < L; ++m) {
                    vv[m] = kInf;
                    RR[m] = 0.0f;
                    EE[m] = 0.0f;
                    if (lid[m] >= 0 && la[m] >= thr) {
                        const float2 cn = p.cnorm[lid[m]];
                        const float sj = xn.y + cn.x;
                        RR[m] = __fadd_ru(__fadd_ru(xn.z, cn.y), __fmul_ru(kCenterEps, sj));
                        EE[m] = __fmul_ru(p.e_coef, __fmul_ru(sj, sj));
                        vv[m] = fmaf(-2.0f, la[m], xn.x) * inv_s2;
                        H = fminf(H, hi_bound(vv[m], EE[m], RR[m], p.g_hi));
                    }
                }
                const bool finite = best > kNegInf && H < kInf && Rmax < kInf && Emax < kInf;
                if (!finite || ovf) {
                    need_full = true;
                } else {
#pragma unroll
                    for (int m = 0; m < L; ++m) {
                        lo[m] = vv[m] < kInf ? lo_bound(vv[m], EE[m], RR[m], p.g_lo) : kInf;
                        if (lo[m] <= H) cmask |= 1u << m;
                    }
                    const int nc = __popc(cmask);
                    if (nc == 0) need_full = true;
                    else if (nc > 1) need_rc = true;
                }
                // Provisional label: the candidate with the largest
                // accumulator (the final one when it is the only candidate;
                // the re-checks overwrite the others).
                float vb = kNegInf;
#pragma unroll
                for (int m = 0; m < L; ++m) {
                    if (((cmask >> m) & 1u) && la[m] > vb) {
                        vb = la[m];
                        jb = lid[m];
                    }
                }
                p.labels[i] = jb;
            }
            // member counts for the centroid update: one reduction per frame
            // (its value unused, so the warp does not wait for it; gathering
            // equal labels of a warp first cost the kernel more than it saved)
            if (p.label_counts && i < p.n) atomicAdd(&p.label_counts[jb], 1);
            const unsigned m_rc = __ballot_sync(0xffffffffu, need_rc);
            if (m_rc) {
                // One entry per re-checked frame and one pair per candidate,
                // both appended with a single atomic per warp.
                const int leader = __ffs(m_rc) - 1;
                const int npairs = need_rc ? __popc(cmask) : 0;
                int excl = npairs;
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const int v = __shfl_up_sync(0xffffffffu, excl, off);
                    if (lane >= off) excl += v;
                }
                const int total = __shfl_sync(0xffffffffu, excl, 31);
                excl -= npairs;
                int base = 0, pbase = 0;
                if (lane == leader) {
                    base = atomicAdd(&p.counters[0], __popc(m_rc));
                    pbase = atomicAdd(&p.counters[2], total);
                }
                base = __shfl_sync(0xffffffffu, base, leader);
                pbase = __shfl_sync(0xffffffffu, pbase, leader);
                if (need_rc) {
                    const int e = base + __popc(m_rc & ((1u << lane) - 1u));
                    // The candidate with the largest accumulator (smallest
                    // approximate distance) is evaluated first; the others are
                    // evaluated only if their lower bound does not exceed it.
                    p.rc_frames[e] = (int32_t)i;
                    p.rc_best[e] = jb;
                    p.rc_keys[e] = ~0ull;
                    p.rc_pairs[e] = ((int64_t)(pbase + excl) << 8) | (int64_t)npairs;
#pragma unroll
                    for (int m = 0; m < L; ++m) {
                        if ((cmask >> m) & 1u) {
                            const int q = pbase + excl + __popc(cmask & ((1u << m) - 1u));
                            p.pair_center[q] = lid[m];
                            p.pair_lo[q] = lo[m];
                        }
                    }
                }
            }
            const unsigned m_full = __ballot_sync(0xffffffffu, need_full);
            if (m_full) {
                const int leader = __ffs(m_full) - 1;
                int base = 0;
                if (lane == leader) base = atomicAdd(&p.counters[1], __popc(m_full));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (need_full) {
                    const int e = base + __popc(m_full & ((1u << lane) - 1u));
                    p.full_frames[e] = (int32_t)i;
                    p.full_keys[e] = ~0ull;
                }
            }
            if (__any_sync(0xffffffffu, *abort_flag != 0)) ok = false;
        }
        if (!ok) {
            atomicOr(p.err, (uint32_t)kDevTimeoutEpi);
            *abort_flag = 1;
        }
        if (pw_acc) {
            atomicAdd(&p.wait_cycles[kWaitEpiAcc], w_acc);
            atomicAdd(&p.wait_cycles[kEpiTotal], (unsigned long long)(clock64() - t_start));
        }
    }

    tc_fence_before();
    __syncthreads();
    // A pair leaves together: no remote arrive or copy may target a CTA that
    // has exited, and the pair's TMEM is released by both CTAs at once.
    if (PAIR) cluster_sync_all();
    if (warp == 1) {
        tc_fence_after();
        if (PAIR)
            tmem_dealloc_pair(tmem_base, p.tmem_cols);
        else
            tmem_dealloc(tmem_base, p.tmem_cols);
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                  CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);

EncodeTiledFn get_encode() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

// Tensor map of an operand (rows x kp elements, row-major): boxes of
// box_rows rows and one 128-byte chunk (64 16-bit or 128 8-bit elements).
int make_map(CUtensorMap *tm, const void *base, int64_t rows, int kp, int box_rows, const TcBuffers &b,
             CUtensorMapSwizzle swizzle) {
    EncodeTiledFn enc = get_encode();
    if (!enc) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return KM_ERR_UNSUPPORTED;
    }
    cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)kp * (cuuint64_t)b.esize};
    cuuint32_t box[2] = {(cuuint32_t)(128 / b.esize), (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    const CUtensorMapDataType dt = b.fp8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                                         : (b.bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16);
    CUresult r = enc(tm, dt, 2,
                     const_cast<void *>(base), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d) for %lld x %d rows/box %d", (int)r, (long long)rows, kp,
                  box_rows);
        return KM_ERR_CUDA;
    }
    return KM_OK;
}

int kp_of(int d) { return (d + 2 + kKC - 1) / kKC * kKC; }
// FP8 rows: the d features in 128-element (128-byte) chunks; no norm columns.
int kp8_of(int d) { return (d + 127) / 128 * 128; }

int pick_bn(int k) {
    if (k >= 256) return 256;
    int bn = (k + 31) / 32 * 32;
    return bn < 32 ? 32 : bn;
}

int k_pad_of(int k) { return (k + 255) / 256 * 256; }

struct Plan {
    int bn, stages, nkc, smem, stream_a;
    int pair;      // CTA-pair form (cta_group::2, M = 256)
    int list_len;  // candidates kept per frame (8 or 16)
    uint32_t tmem_cols;
};

// Tile shapes chosen by km_tune_tiles, per (d, k), and the shape a tuning
// thread forces while it times the candidates.
struct PlanTable {
    std::mutex m;
    std::map<std::pair<int, int>, TilePlan> choice;
} g_plans;
thread_local const TilePlan *t_forced_plan = nullptr;

// The CTA-pair form is used for full-width center tiles with a resident frame
// tile; KM_TC_PAIR=0 or 1 in the environment forces the choice (both forms
// give the same labels).
bool pair_wanted() {
    const char *e = std::getenv("KM_TC_PAIR");
    if (e && e[0] == '0') return false;
    return true;
}

// The plan of a given tile shape: bn columns per center tile (a multiple of
// 32, at most 256), the CTA-pair form (bn = 256, resident frame tile only),
// max_stages caps the TMA ring (0: as many as fit).  False when the shape
// does not fit.
bool build_plan(int d, int bn, bool pair, int max_stages, int list_len, Plan &pl, bool fp8 = false) {
    if (bn < 32 || bn > 256 || bn % 32 || (list_len != 8 && list_len != 16)) return false;
    pl.nkc = fp8 ? kp8_of(d) / 128 : kp_of(d) / kKC;
    pl.bn = bn;
    pl.list_len = list_len;
    pl.stream_a = 0;
    pl.pair = 0;
    const int cap = max_stages > 0 ? std::min(8, max_stages) : 8;
    const int fixed = 1024 + 512;
    int stages = 0;
    if (pl.nkc <= kMaxNkc) {
        const int res = fixed + pl.nkc * kABytesPerChunk;
        if (pair) {
            // Each CTA of the pair stages half of the B tile: 16 KB per stage.
            if (bn != 256) return false;
            const int half = pl.bn / 2 * kKC * 2;
            stages = std::min(cap, (kSmemLimit - res) / half);
            if (stages < 3) return false;
            pl.pair = 1;
            pl.smem = res + stages * half;
        } else {
            stages = std::min(cap, (kSmemLimit - res) / (pl.bn * kKC * 2));
            if (stages >= 2) pl.smem = res + stages * pl.bn * kKC * 2;
        }
    } else if (pair) {
        return false;
    }
    if (stages < 2) {
        // Streaming: each stage carries an A chunk and a full-width B chunk.
        pl.stream_a = 1;
        stages = std::min(cap, (kSmemLimit - fixed) / (kABytesPerChunk + pl.bn * kKC * 2));
        if (stages < 2) return false;
        pl.smem = fixed + stages * (kABytesPerChunk + pl.bn * kKC * 2);
    }
    pl.stages = stages;
    if (pl.smem < 120 * 1024) pl.smem = 120 * 1024;  // one CTA per SM: TMEM is sized for one
    uint32_t cols = 32;
    while (cols < (uint32_t)(2 * pl.bn)) cols <<= 1;
    pl.tmem_cols = cols;
    return true;
}

// The default shape: full-width center tiles (256 columns, or k rounded up
// to 32), the CTA pair where it applies, as many stages as fit, 8 candidates
// (FP16 up to d = 256) or 16.  A shape forced by the tuning thread, or
// stored by km_tune_tiles for (d, k), replaces it.
bool make_plan(int d, int k, Plan &pl, bool fp8 = false, bool bf16 = false) {
    const TilePlan *tp = t_forced_plan;
    TilePlan stored;
    if (!tp) {
        std::lock_guard<std::mutex> lk(g_plans.m);
        auto it = g_plans.choice.find(std::make_pair(d, k));
        if (it != g_plans.choice.end()) {
            stored = it->second;
            tp = &stored;
        }
    }
    if (tp) {
        // (the FP8 kernel keeps 16 candidates)
        if (tp->bn <= pick_bn(k) &&
            build_plan(d, tp->bn, tp->pair != 0, tp->stages, fp8 ? kL : tp->list_len, pl, fp8))
            return true;
        if (t_forced_plan) return false;
    }
    const int bn = pick_bn(k);
    // FP16: 8 candidates up to d = 256, 16 above: km_tune_tiles picked 8 on
    // every measured shape with d <= 256 (fewer list shifts in the epilogue);
    // at d = 528, k = 2000 8 candidates are 20% slower (more lists overflow
    // to the re-check over all centers), at d = 1024 the two tie.  BF16 and
    // FP8 keep 16: their wider bounds leave
    // more candidates per frame (BF16 with 8 at d = 256, k = 5000: 4.3 ->
    // 24.9 ms per iteration, most frames re-checked over all centers).
    const int len = !fp8 && !bf16 && d <= 256 ? 8 : kL;
    if (bn == 256 && pair_wanted() && build_plan(d, bn, true, 0, len, pl, fp8)) return true;
    return build_plan(d, bn, false, 0, len, pl, fp8);
}

bool device_is_sm10x() {
    static int cc[kDeviceSlots] = {};  // compute capability major + 1 (0: not read yet)
    const int dev = current_device();
    if (dev >= 0 && dev < kDeviceSlots && cc[dev]) return cc[dev] == 11;
    int major = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    if (dev >= 0 && dev < kDeviceSlots) cc[dev] = major + 1;
    return major == 10;
}

float norm_inflate_of(int d) {
    // A compensated float32 sum of d squares is within a few u of the true value.
    return 1.0f + (float)(d + 8) * 5.9604645e-8f + 1e-6f;
}

int64_t prep_blocks(int64_t rows) {
    int64_t blocks = (rows * 32 + 255) / 256;
    const int64_t cap = (int64_t)num_sms() * 16;
    if (blocks > cap) blocks = cap;
    return blocks < 1 ? 1 : blocks;
}

}  // namespace

bool tc_plan_exists(int d, int k) {
    Plan pl;
    return make_plan(d, k, pl);
}

void tc_enumerate_plans(int d, int k, std::vector<TilePlan> &out) {
    out.clear();
    const int bn_max = pick_bn(k);
    for (int bn : {256, 128, 64}) {
        if (bn > bn_max) continue;
        for (int pair = 1; pair >= 0; --pair) {
            Plan full;
            if (!build_plan(d, bn, pair != 0, 0, kL, full)) continue;
            // the fullest ring, and shallower ones down to two (three for pairs)
            std::vector<int> st = {full.stages};
            for (int q : {4, 3, 2})
                if (q < full.stages && (pair == 0 || q >= 3)) st.push_back(q);
            for (int q : st)
                for (int len : {16, 8}) {
                    Plan pl;
                    if (build_plan(d, bn, pair != 0, q, len, pl)) out.push_back(TilePlan{bn, pair, pl.stages, len});
                }
        }
    }
    if (bn_max < 64) {
        Plan pl;
        for (int len : {16, 8})
            if (build_plan(d, bn_max, false, 0, len, pl)) out.push_back(TilePlan{bn_max, 0, pl.stages, len});
    }
}

void tc_force_plan(const TilePlan *plan) { t_forced_plan = plan; }

void tc_store_plan(int d, int k, const TilePlan &plan) {
    std::lock_guard<std::mutex> lk(g_plans.m);
    g_plans.choice[std::make_pair(d, k)] = plan;
}

void tc_clear_plans() {
    std::lock_guard<std::mutex> lk(g_plans.m);
    g_plans.choice.clear();
}

bool tc_current_plan(int d, int k, TilePlan *out, bool *tuned) {
    Plan pl;
    if (!make_plan(d, k, pl)) return false;
    *out = TilePlan{pl.bn, pl.pair, pl.stages, pl.list_len};
    std::lock_guard<std::mutex> lk(g_plans.m);
    *tuned = g_plans.choice.count(std::make_pair(d, k)) > 0;
    return true;
}

bool tc_supported(int d, int k) {
    Plan pl;
    return make_plan(d, k, pl) && device_is_sm10x();
}

size_t tc_frames_ws_size(int64_t n, int d) {
    Carver c(nullptr);
    c.take<uint16_t>((size_t)(n > 0 ? n : 1) * kp_of(d));
    c.take<float4>(n > 0 ? n : 1);
    return c.bytes();
}

void tc_carve_frames(void *ws, int64_t n, int d, TcBuffers &b) {
    Carver c(ws);
    b.kp = kp_of(d);
    b.xh = c.take<uint16_t>((size_t)(n > 0 ? n : 1) * b.kp);
    b.xnorm = c.take<float4>(n > 0 ? n : 1);
}

size_t tc_centers_ws_size(int d, int k) {
    Carver c(nullptr);
    c.take<uint16_t>((size_t)k_pad_of(k) * kp_of(d));
    c.take<float2>(k_pad_of(k));
    c.take<float>(d);
    c.take<uint32_t>(kNumScalars);
    c.take<float>(k_pad_of(k));
    return c.bytes();
}

void tc_carve_centers(void *ws, int d, int k, TcBuffers &b) {
    Carver c(ws);
    b.kp = kp_of(d);
    b.ch = c.take<uint16_t>((size_t)k_pad_of(k) * b.kp);
    b.cnorm = c.take<float2>(k_pad_of(k));
    b.shift = c.take<float>(d);
    b.scal = c.take<uint32_t>(kNumScalars);
    b.chn = c.take<float>(k_pad_of(k));
}

// The 16-bit buffers hold kp_of(d) 2-byte elements per row; an FP8 row of
// kp8_of(d) bytes fits in them.
void tc_set_operand(TcBuffers &b, int d, int prec) {
    b.bf16 = prec == KM_PREC_BF16;
    b.fp8 = prec == KM_PREC_FP8;
    b.esize = b.fp8 ? 1 : 2;
    b.kp = b.fp8 ? kp8_of(d) : kp_of(d);
}

namespace {
// A deferred pass (tc_assign_deferred) runs in up to kMaxTcChunks launches
// over consecutive frame ranges; chunk c's candidate lists start at the
// chunk's first frame (an entry per frame at most), its counters at
// kChunkCounters0 + 4 (c - 1) (chunk 0 uses counters[0..4)).
constexpr int kMaxTcChunks = kTcMaxChunks;
constexpr int kChunkCounters0 = 20;

// One carving sequence for sizing (ws == nullptr) and for carving.
size_t carve_assign(void *ws, int64_t n, TcBuffers &b) {
    Carver c(ws);
    const size_t nn = n > 0 ? n : 1;
    b.rc_frames = c.take<int32_t>(nn);
    b.pair_center = c.take<int32_t>(nn * kL);
    b.rc_keys = c.take<unsigned long long>(nn);
    b.rc_best = c.take<int32_t>(nn);
    b.pair_lo = c.take<float>(nn * kL);
    b.rc_pairs = c.take<int64_t>(nn);
    b.amb_entries = c.take<int32_t>(nn);
    b.amb_mask = c.take<int32_t>(nn);
    b.full_frames = c.take<int32_t>(nn);
    b.full_keys = c.take<unsigned long long>(nn);
    // [0] recheck entries, [1] full entries, [2] pairs, [3] entries left to the exact pass, [4..20) diagnostics,
    // then the same four for chunks 1.. of a chunked pass
    b.counters = c.take<int32_t>(kChunkCounters0 + 4 * (kMaxTcChunks - 1));
    b.flipped = c.take<unsigned long long>(1);
    b.err = c.take<uint32_t>(1);
    return c.bytes();
}
}  // namespace

size_t tc_assign_ws_size(int64_t n, int d, int k) {
    (void)d;
    (void)k;
    TcBuffers b;
    return carve_assign(nullptr, n, b);
}

void tc_carve_assign(void *ws, int64_t n, int d, int k, TcBuffers &b) {
    (void)d;
    (void)k;
    carve_assign(ws, n, b);
}

int tc_prepare_shift_from_centers(const float *C, int d, int k, TcBuffers &b, cudaStream_t s) {
    shift_mean_kernel<<<(d + 31) / 32, kShiftWarps * 32, 0, s>>>(C, d, k, b.shift);
    KM_CUDA(cudaGetLastError());
    KM_CUDA(cudaMemsetAsync(b.scal, 0, kNumScalars * sizeof(uint32_t), s));
    if (b.fp8) {
        center_absmax_kernel<<<(unsigned)prep_blocks(k), 256, 0, s>>>(C, k, d, b.shift, b.scal);
        KM_CUDA(cudaGetLastError());
        scale_fp8_finalize_kernel<<<1, 1, 0, s>>>(b.scal);
    } else {
        center_norm_max_kernel<<<(unsigned)prep_blocks(k), 256, 0, s>>>(C, k, d, b.shift, b.scal);
        KM_CUDA(cudaGetLastError());
        scale_finalize_kernel<<<1, 1, 0, s>>>(b.scal);
    }
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

template <typename T, int IT>
void launch_prep_v4(const float *X, int64_t n, int d, TcBuffers &b, cudaStream_t s) {
    prep_frames_v4_kernel<T, IT><<<(unsigned)prep_blocks(n), 256, 0, s>>>(X, n, d, b.kp, b.shift, b.scal,
                                                                        reinterpret_cast<T *>(b.xh), b.xnorm,
                                                                        norm_inflate_of(d));
}

template <typename T>
void prepare_frames_t(const float *X, int64_t n, int d, TcBuffers &b, cudaStream_t s) {
    const int it = (b.kp + 127) / 128;
    const bool v4 = d % 4 == 0 && it <= 9 &&
                    ((reinterpret_cast<uintptr_t>(X) | reinterpret_cast<uintptr_t>(b.shift)) & 15) == 0;
    if (v4) {
        switch (it) {
            case 1: launch_prep_v4<T, 1>(X, n, d, b, s); break;
            case 2: launch_prep_v4<T, 2>(X, n, d, b, s); break;
            case 3: launch_prep_v4<T, 3>(X, n, d, b, s); break;
            case 4: launch_prep_v4<T, 4>(X, n, d, b, s); break;
            case 5: launch_prep_v4<T, 5>(X, n, d, b, s); break;
            case 6: launch_prep_v4<T, 6>(X, n, d, b, s); break;
            case 7: launch_prep_v4<T, 7>(X, n, d, b, s); break;
            case 8: launch_prep_v4<T, 8>(X, n, d, b, s); break;
            default: launch_prep_v4<T, 9>(X, n, d, b, s); break;
        }
    } else {
        prep_frames_kernel<T><<<(unsigned)prep_blocks(n), 256, 0, s>>>(DenseRows{X, d}, n, d, b.kp, b.shift, b.scal,
                                                                     reinterpret_cast<T *>(b.xh), b.xnorm,
                                                                     norm_inflate_of(d));
    }
}

int tc_prepare_frames(const float *X, int64_t n, int d, TcBuffers &b, cudaStream_t s, const PairSrc *ps) {
    if (n == 0) return KM_OK;
    if (ps) {
        // pair features computed in the conversion: no float32 copy of them
        if (b.fp8) {
            set_error("FP8 operands are not built for coordinate frames");
            return KM_ERR_UNSUPPORTED;
        }
        const PairRows pr{ps->xyz, reinterpret_cast<const int2 *>(ps->pairs), ps->n_atoms, d};
        const size_t smem = prep_pairs_smem(d, ps->n_atoms);
        if (ps->n_atoms <= kPrepPairMaxAtoms && smem <= 48 * 1024) {
            if (b.bf16)
                prep_frames_pairs_kernel<__nv_bfloat16><<<(unsigned)prep_blocks(n), kPrepPairThreads, smem, s>>>(
                    pr, n, d, b.kp, b.shift, b.scal, reinterpret_cast<__nv_bfloat16 *>(b.xh), b.xnorm,
                    norm_inflate_of(d));
            else
                prep_frames_pairs_kernel<__half><<<(unsigned)prep_blocks(n), kPrepPairThreads, smem, s>>>(
                    pr, n, d, b.kp, b.shift, b.scal, reinterpret_cast<__half *>(b.xh), b.xnorm, norm_inflate_of(d));
            KM_CUDA(cudaGetLastError());
            return KM_OK;
        }
        if (b.bf16)
            prep_frames_kernel<__nv_bfloat16><<<(unsigned)prep_blocks(n), 256, 0, s>>>(
                pr, n, d, b.kp, b.shift, b.scal, reinterpret_cast<__nv_bfloat16 *>(b.xh), b.xnorm, norm_inflate_of(d));
        else
            prep_frames_kernel<__half><<<(unsigned)prep_blocks(n), 256, 0, s>>>(
                pr, n, d, b.kp, b.shift, b.scal, reinterpret_cast<__half *>(b.xh), b.xnorm, norm_inflate_of(d));
        KM_CUDA(cudaGetLastError());
        return KM_OK;
    }
    if (b.fp8)
        prep_frames_fp8_kernel<<<(unsigned)prep_blocks(n), 256, 0, s>>>(
            X, n, d, b.kp, b.shift, b.scal, static_cast<uint8_t *>(b.xh), b.xnorm, norm_inflate_of(d));
    else if (b.bf16)
        prepare_frames_t<__nv_bfloat16>(X, n, d, b, s);
    else
        prepare_frames_t<__half>(X, n, d, b, s);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

int tc_prepare_centers(const float *C, int d, int k, TcBuffers &b, cudaStream_t s) {
    const int kpad = k_pad_of(k);
    KM_CUDA(cudaMemsetAsync(b.scal + kCmax, 0, 2 * sizeof(uint32_t), s));  // kCmax, kHcMax
    KM_CUDA(cudaMemsetAsync(b.ch, 0, (size_t)kpad * b.kp * b.esize, s));
    if (b.fp8)
        prep_centers_fp8_kernel<<<(unsigned)prep_blocks(kpad), 256, 0, s>>>(
            C, k, kpad, d, b.kp, b.shift, b.scal, static_cast<uint8_t *>(b.ch), b.cnorm, b.chn, norm_inflate_of(d));
    else if (b.bf16)
        prep_centers_kernel<__nv_bfloat16><<<(unsigned)prep_blocks(kpad), 256, 0, s>>>(
            C, k, kpad, d, b.kp, b.shift, b.scal, reinterpret_cast<__nv_bfloat16 *>(b.ch), b.cnorm,
            norm_inflate_of(d));
    else
        prep_centers_kernel<__half><<<(unsigned)prep_blocks(kpad), 256, 0, s>>>(
            C, k, kpad, d, b.kp, b.shift, b.scal, reinterpret_cast<__half *>(b.ch), b.cnorm, norm_inflate_of(d));
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

namespace {

constexpr int kRecheckBesidePerSm = 4;

// The launches of a pass over frames [0, n): one, or with a side stream and
// n_fork > 1 fork events, consecutive ranges of at least 256k frames each
// (KM_TC_CHUNKS sets the number, default 4), so that chunk c's re-check runs
// beside the tensor-core launch of chunk c + 1.
int tc_chunks_for(int64_t n, int n_fork) {
    if (n_fork <= 1) return 1;
    int want = 4;
    if (const char *e = std::getenv("KM_TC_CHUNKS")) want = std::atoi(e);
    want = std::max(1, std::min(want, std::min(n_fork, kMaxTcChunks)));
    const int64_t by_size = n >> 18;
    if (want > by_size) want = (int)std::max<int64_t>(1, by_size);
    return want;
}

// First frame of chunk c (of n_chunks) over n frames: a multiple of `wave`
// (the frames one launch's CTAs take in one round of units, a multiple of
// 256) where a chunk holds at least one wave, so that every chunk but the
// last ends without a partial round; else a multiple of 256.
int64_t chunk_first(int64_t n, int n_chunks, int c, int64_t wave) {
    if (c >= n_chunks) return n;
    const int64_t step = n / n_chunks >= wave ? wave : 256;
    return (n / n_chunks * c + step / 2) / step * step;
}

// Candidate lists and counters of chunk c, which starts at frame a.
void chunk_lists(const TcBuffers &b, int64_t a, int c, TcBuffers &v) {
    v = b;
    if (c == 0) return;
    v.rc_frames = b.rc_frames + a;
    v.pair_center = b.pair_center + a * kL;
    v.rc_keys = b.rc_keys + a;
    v.rc_best = b.rc_best + a;
    v.pair_lo = b.pair_lo + a * kL;
    v.rc_pairs = b.rc_pairs + a;
    v.amb_entries = b.amb_entries + a;
    v.amb_mask = b.amb_mask + a;
    v.full_frames = b.full_frames + a;
    v.full_keys = b.full_keys + a;
    v.counters = b.counters + kChunkCounters0 + 4 * (c - 1);
}

void set_lists(TcParams &p, const TcBuffers &v) {
    p.rc_frames = v.rc_frames;
    p.pair_center = v.pair_center;
    p.rc_keys = v.rc_keys;
    p.rc_best = v.rc_best;
    p.rc_pairs = v.rc_pairs;
    p.pair_lo = v.pair_lo;
    p.full_frames = v.full_frames;
    p.full_keys = v.full_keys;
    p.counters = v.counters;
}

template <bool PAIR>
cudaError_t launch_tc_variant(const cudaLaunchConfig_t &cfg, int list_len, bool fp8, const CUtensorMap &tmA,
                              const CUtensorMap &tmB, const TcParams &p) {
    if (fp8) return cudaLaunchKernelEx(&cfg, tc_assign_kernel<PAIR, 16, true>, tmA, tmB, p);
    if (list_len == 8) return cudaLaunchKernelEx(&cfg, tc_assign_kernel<PAIR, 8, false>, tmA, tmB, p);
    return cudaLaunchKernelEx(&cfg, tc_assign_kernel<PAIR, 16, false>, tmA, tmB, p);
}

int tc_assign_impl(const float *X, int64_t n, int d, const float *C, int k, int32_t *labels, TcBuffers &b,
                   cudaStream_t s, ProfEvents *prof, float *dump, unsigned long long *wait_cycles, cudaStream_t side,
                   const cudaEvent_t *ev_fork, int n_fork, const FlipList *fl, const PairSrc *ps,
                   int32_t *label_counts) {
    if (n == 0) return KM_OK;
    Plan pl;
    if (!make_plan(d, k, pl, b.fp8 != 0, b.bf16 != 0) || !device_is_sm10x()) {
        set_error("no tensor-core plan for d=%d k=%d on this device", d, k);
        return KM_ERR_UNSUPPORTED;
    }
    {
        // The shared-memory opt-in holds per device: set it once on each.
        static std::mutex attr_mu;
        static bool attr_done[kDeviceSlots] = {};
        const int dev = current_device();
        std::lock_guard<std::mutex> lk(attr_mu);
        if (dev < 0 || dev >= kDeviceSlots || !attr_done[dev]) {
            const void *fns[6] = {(const void *)tc_assign_kernel<false, 16, false>,
                                  (const void *)tc_assign_kernel<true, 16, false>,
                                  (const void *)tc_assign_kernel<false, 8, false>,
                                  (const void *)tc_assign_kernel<true, 8, false>,
                                  (const void *)tc_assign_kernel<false, 16, true>,
                                  (const void *)tc_assign_kernel<true, 16, true>};
            for (const void *f : fns)
                KM_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemLimit));
            if (dev >= 0 && dev < kDeviceSlots) attr_done[dev] = true;
        }
    }
    // (the FP8 kernel keeps 16 candidates: make_plan set list_len)
    const void *kfn = b.fp8 ? (pl.pair ? (const void *)tc_assign_kernel<true, 16, true>
                                       : (const void *)tc_assign_kernel<false, 16, true>)
                            : pl.pair ? (pl.list_len == 8 ? (const void *)tc_assign_kernel<true, 8, false>
                                                          : (const void *)tc_assign_kernel<true, 16, false>)
                                      : (pl.list_len == 8 ? (const void *)tc_assign_kernel<false, 8, false>
                                                          : (const void *)tc_assign_kernel<false, 16, false>);

    CUtensorMap tmA, tmB;
    KM_TRY(make_map(&tmA, b.xh, n, b.kp, kBM, b, CU_TENSOR_MAP_SWIZZLE_128B));
    KM_TRY(make_map(&tmB, b.ch, k_pad_of(k), b.kp, pl.pair ? pl.bn / 2 : pl.bn, b, CU_TENSOR_MAP_SWIZZLE_128B));

    const int n_chunks = side ? tc_chunks_for(n, n_fork) : 1;
    KM_CUDA(cudaMemsetAsync(b.counters, 0, 4 * sizeof(int32_t), s));
    if (n_chunks > 1)
        KM_CUDA(cudaMemsetAsync(b.counters + kChunkCounters0, 0, 4 * (size_t)(n_chunks - 1) * sizeof(int32_t), s));
    KM_CUDA(cudaMemsetAsync(b.flipped, 0, sizeof(unsigned long long), s));
    if (!b.keep_err) KM_CUDA(cudaMemsetAsync(b.err, 0, sizeof(uint32_t), s));

    const double u = 5.9604644775390625e-08;  // 2^-24
    TcParams p;
    p.n = n;
    p.frame0 = 0;
    p.label_counts = label_counts;
    p.k = k;
    p.d = d;
    p.kp = b.kp;
    p.nkc = pl.nkc;
    // K steps holding data: 16 elements (d features and two norm columns) in
    // the 16-bit forms, 32 elements (d features) in FP8.
    p.ksteps_total = b.fp8 ? (d + 31) / 32 : (d + 2 + 15) / 16;
    p.stream_a = pl.stream_a;
    p.nbst = (p.ksteps_total + 3) / 4;
    p.bn = pl.bn;
    p.stages = pl.stages;
    p.n_ctiles = (k + pl.bn - 1) / pl.bn;
    p.tmem_cols = pl.tmem_cols;
    const double gamma_acc = (b.kp / 16 + 1) * std::ldexp(1.0, -21);
    // The hi/lo split of -||c_hat||^2/2 leaves at most 2^-24 (FP16) or 2^-18
    // (BF16) of it; the bound allows 2^-21 and 2^-17.
    p.bf16 = b.bf16;
    p.e_coef = (float)((gamma_acc * 1.003 + std::ldexp(1.0, b.bf16 ? -17 : -21) + 8.0 * u) * 1.01);
    if (b.fp8) {
        // FP8: the accumulation of the e4m3 products in the MMA (its internal
        // precision is not published; the allowance is 2^-18 of the row norms
        // per 32-element K step, 8 times the FP16 form's per-step allowance,
        // and the bound test measures the share the hardware uses), the
        // epilogue's fused multiply-add and the rounded norms ||x~||^2 and
        // ||c~||^2 / 2 (16 u of (sx + sc)^2 in all).
        p.e_coef = (float)((2.0 * p.ksteps_total * std::ldexp(1.0, -18) + 16.0 * u) * 1.25);
    }
    const double g = (d + 2) * u / (1.0 - (d + 2) * u) * 1.01;
    p.g_lo = (float)((1.0 - g) * (1.0 - 4.0 * u));
    p.g_hi = (float)((1.0 + g) * (1.0 + 4.0 * u));
    // sqrt(g_hi / g_lo) of the float factors, inflated by 2^-19 and rounded up.
    p.g_ratio = std::nextafter((float)(std::sqrt((double)p.g_hi / (double)p.g_lo) * (1.0 + std::ldexp(1.0, -19))),
                               INFINITY);
    p.xnorm = b.xnorm;
    p.cnorm = b.cnorm;
    p.chn = b.chn;
    p.scal = b.scal;
    p.labels = labels;
    // Seeds for 16-bit operands with short rows and many center tiles: there
    // the candidate lists of a frame's first tiles are a large part of the
    // epilogue's work, and a seed costs two rows of at most 256 bytes per
    // frame (1M frames, d = 16 and 64, k = 5000: 10-15% faster iterations;
    // k = 1000, four tiles: no gain, and 2.5% slower at d = 10).
    // KM_TC_SEED=0 or 1 in the environment forces the choice for 16-bit
    // operands (both give the same labels).
    bool seed = !b.fp8 && b.kp <= 128 && k >= 2048;
    if (const char *e = std::getenv("KM_TC_SEED")) seed = !b.fp8 && e[0] == '1';
    p.seed_xh = seed ? b.xh : nullptr;
    p.seed_ch = seed ? b.ch : nullptr;
    {
        const double uu = std::ldexp(1.0, -24);
        const double kk = (double)b.kp + 2.0;
        p.seed_coef = std::nextafter((float)(kk * uu / (1.0 - kk * uu) * 1.01), INFINITY);
    }
    set_lists(p, b);
    p.err = b.err;
    p.dump = dump;
    p.wait_cycles = wait_cycles;

    // The launches of a chunked pass run at the device's greatest priority:
    // when a chunk ends, the next chunk's CTAs are placed before the CTAs of
    // the re-check that waits for it.  The kernel walks its frame units in a
    // fixed order per CTA, so one CTA placed late would delay its launch; the
    // re-check beside it takes one CTA per SM, which fits next to a
    // tensor-core CTA (no shared memory, few registers).
    int prio = 0;
    if (n_chunks > 1) {
        int least = 0;
        KM_CUDA(cudaDeviceGetStreamPriorityRange(&least, &prio));
    }
    // CTA pairs: as many clusters of two CTAs as fit at once (one CTA per
    // SM), each walking 256-frame units.
    int clusters_fit = 0;
    if (pl.pair) {
        static std::mutex cl_mu;
        // (device, shared memory, list length, FP8) -> clusters
        static std::map<std::tuple<int, int, int, int>, int> cached_clusters;
        const auto key = std::make_tuple(current_device(), pl.smem, pl.list_len, b.fp8 != 0 ? 1 : 0);
        std::lock_guard<std::mutex> lk(cl_mu);
        auto it = cached_clusters.find(key);
        if (it == cached_clusters.end()) {
            cudaLaunchConfig_t qc = {};
            cudaLaunchAttribute qa[1];
            qa[0].id = cudaLaunchAttributeClusterDimension;
            qa[0].val.clusterDim.x = 2;
            qa[0].val.clusterDim.y = 1;
            qa[0].val.clusterDim.z = 1;
            qc.blockDim = dim3(kThreadsTC, 1, 1);
            qc.dynamicSmemBytes = (size_t)pl.smem;
            qc.stream = s;
            qc.attrs = qa;
            qc.numAttrs = 1;
            qc.gridDim = dim3((unsigned)(2 * (num_sms() / 2)), 1, 1);
            int nc = 0;
            KM_CUDA(cudaOccupancyMaxActiveClusters(&nc, kfn, &qc));
            it = cached_clusters.emplace(key, nc).first;
        }
        clusters_fit = it->second;
        if (clusters_fit < 1) {
            set_error("no CTA pair of the tensor-core kernel fits on this device");
            return KM_ERR_UNSUPPORTED;
        }
    }
    // Frames one launch takes in one round of units over all its CTAs.
    const int64_t wave = pl.pair ? 2 * kBM * (int64_t)clusters_fit : kBM * (int64_t)num_sms();
    auto launch_pass = [&](const TcParams &q) -> int {
        const int64_t rows = q.n - q.frame0;
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[2];
        int na = 0;
        cfg.blockDim = dim3(kThreadsTC, 1, 1);
        cfg.dynamicSmemBytes = (size_t)pl.smem;
        cfg.stream = s;
        cfg.attrs = attr;
        if (pl.pair) {
            attr[na].id = cudaLaunchAttributeClusterDimension;
            attr[na].val.clusterDim.x = 2;
            attr[na].val.clusterDim.y = 1;
            attr[na].val.clusterDim.z = 1;
            ++na;
            const int64_t n_units = (rows + 2 * kBM - 1) / (2 * kBM);
            int64_t clusters = clusters_fit;
            if (clusters > n_units) clusters = n_units;
            cfg.gridDim = dim3((unsigned)(2 * clusters), 1, 1);
        } else {
            const int64_t n_ftiles = (rows + kBM - 1) / kBM;
            int64_t grid = num_sms();
            if (grid > n_ftiles) grid = n_ftiles;
            cfg.gridDim = dim3((unsigned)grid, 1, 1);
        }
        if (n_chunks > 1) {
            attr[na].id = cudaLaunchAttributePriority;
            attr[na].val.priority = prio;
            ++na;
        }
        cfg.numAttrs = na;
        KM_CUDA(pl.pair ? launch_tc_variant<true>(cfg, pl.list_len, b.fp8 != 0, tmA, tmB, q)
                        : launch_tc_variant<false>(cfg, pl.list_len, b.fp8 != 0, tmA, tmB, q));
        KM_CUDA(cudaGetLastError());
        return KM_OK;
    };

    // Each chunk: the tensor-core launch on s, then its exact re-checks on s,
    // or on `side` beside the next chunk (and, after the last chunk, beside
    // the caller's next work).  Beside the centroid update the re-check keeps
    // to half of each SM's threads, beside a tensor-core launch to one CTA
    // per SM, so that both stay resident.
    cudaStream_t r = side ? side : s;
    if (prof) prof->begin(kProfTc, s);
    int64_t f_next = 0;
    for (int c = 0; c < n_chunks; ++c) {
        const int64_t f0 = f_next;
        TcBuffers v;
        chunk_lists(b, f0, c, v);
        TcParams q = p;
        q.frame0 = f0;
        q.n = n;
        if (c + 1 < n_chunks) q.n = std::min(n, std::max(f0 + 256, chunk_first(n, n_chunks, c + 1, wave)));
        const int64_t f1 = q.n;
        f_next = f1;
        set_lists(q, v);
        KM_TRY(launch_pass(q));
        if (prof && c + 1 == n_chunks) prof->end(kProfTc, s);
        if (side) {
            KM_CUDA(cudaEventRecord(ev_fork[c], s));
            KM_CUDA(cudaStreamWaitEvent(side, ev_fork[c], 0));
        }
        if (prof && c == 0) prof->begin(kProfRecheck, r);
        const int per_sm = !side ? 8 : c + 1 < n_chunks ? 1 : kRecheckBesidePerSm;
        KM_TRY(launch_recheck_pairs(X, d, C, v.rc_frames, v.rc_best, v.rc_pairs, v.pair_center, v.pair_lo,
                                    v.rc_keys, v.amb_entries, v.amb_mask, v.counters, f1 - f0, labels, b.flipped, r,
                                    fl, per_sm, ps));
        if (n_chunks > 1)
            KM_TRY(launch_full_recheck(X, v.full_frames, v.counters + 1, f1 - f0, d, C, k, v.full_keys, labels,
                                       b.flipped, r, fl, ps));
    }
    if (prof) prof->end(kProfRecheck, r);
    if (n_chunks == 1) {
        if (prof) prof->begin(kProfFull, r);
        KM_TRY(launch_full_recheck(X, b.full_frames, b.counters + 1, n, d, C, k, b.full_keys, labels, b.flipped, r,
                                   fl, ps));
        if (prof) prof->end(kProfFull, r);
    }
    return KM_OK;
}

}  // namespace

int tc_assign(const float *X, int64_t n, int d, const float *C, int k, int32_t *labels, TcBuffers &b,
              cudaStream_t s, ProfEvents *prof, float *dump, unsigned long long *wait_cycles, const PairSrc *ps) {
    return tc_assign_impl(X, n, d, C, k, labels, b, s, prof, dump, wait_cycles, nullptr, nullptr, 0, nullptr, ps,
                          nullptr);
}

int tc_assign_deferred(const float *X, int64_t n, int d, const float *C, int k, int32_t *labels, TcBuffers &b,
                       cudaStream_t s, cudaStream_t side, const cudaEvent_t *ev_fork, int n_fork, const FlipList &fl,
                       ProfEvents *prof, const PairSrc *ps, int32_t *label_counts) {
    return tc_assign_impl(X, n, d, C, k, labels, b, s, prof, nullptr, nullptr, side, ev_fork, n_fork, &fl, ps,
                          label_counts);
}

}  // namespace km

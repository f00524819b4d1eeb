// km_common.cuh -- shared helpers of libkmgpu: status plumbing, workspace
// carving, exact float32 distance, Philox4x32-10 and bounded device waits.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>

#include "../../include/kmgpu.h"

namespace km {

// ---------------------------------------------------------------------------
// Error reporting (thread-local message, see km_last_error()).
// ---------------------------------------------------------------------------
void set_error(const char *fmt, ...);

inline int cuda_fail(cudaError_t e, const char *what) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return KM_ERR_CUDA;
}

#define KM_CUDA(call)                                          \
    do {                                                       \
        cudaError_t _e = (call);                               \
        if (_e != cudaSuccess) return ::km::cuda_fail(_e, #call); \
    } while (0)

#define KM_TRY(call)                \
    do {                            \
        int _s = (call);            \
        if (_s != KM_OK) return _s; \
    } while (0)

// ---------------------------------------------------------------------------
// Workspace carving: sub-buffers aligned to 256 bytes.  The same sequence of
// take() calls is run once with base == nullptr to size the workspace.
// ---------------------------------------------------------------------------
struct Carver {
    char *base;
    size_t off = 0;
    explicit Carver(void *b) : base(static_cast<char *>(b)) {}
    template <typename T>
    T *take(size_t count) {
        off = (off + 255) & ~size_t(255);
        T *p = base ? reinterpret_cast<T *>(base + off) : nullptr;
        off += count * sizeof(T);
        return p;
    }
    size_t bytes() const { return (off + 255) & ~size_t(255); }
};

constexpr int kMaxD = 4096;
constexpr int kMaxK = 1 << 20;

inline int check_shape(int64_t n, int32_t d, int32_t k) {
    if (n < 0 || n >= (int64_t(1) << 31)) {
        set_error("n=%lld out of range [0, 2^31)", (long long)n);
        return KM_ERR_BAD_SHAPE;
    }
    if (d < 1 || d > kMaxD) {
        set_error("d=%d out of range [1, %d]", d, kMaxD);
        return KM_ERR_BAD_SHAPE;
    }
    if (k < 1 || k > kMaxK) {
        set_error("k=%d out of range [1, %d]", k, kMaxK);
        return KM_ERR_BAD_SHAPE;
    }
    return KM_OK;
}

inline int check_ws(void *ws, size_t have, size_t need) {
    if (need == 0) return KM_OK;
    if (!ws || have < need) {
        set_error("workspace of %zu bytes given, %zu needed", have, need);
        return KM_ERR_WORKSPACE;
    }
    return KM_OK;
}

// Per-device caches (function attributes, occupancy, SM counts) are indexed
// by the current device's ordinal; ordinals from kDeviceSlots on are queried
// each time.
constexpr int kDeviceSlots = 64;

inline int current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        dev = 0;
    }
    return dev;
}

inline int num_sms() {
    static int cached[kDeviceSlots] = {};
    const int dev = current_device();
    if (dev >= 0 && dev < kDeviceSlots && cached[dev]) return cached[dev];
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    v = v > 0 ? v : 1;
    if (dev >= 0 && dev < kDeviceSlots) cached[dev] = v;
    return v;
}

// Device error word written by kernels whose waits ran out (bit set per site).
enum DeviceError : uint32_t {
    kDevTimeoutTma = 1u,
    kDevTimeoutMma = 2u,
    kDevTimeoutEpi = 4u,
    kDevBadLabel = 8u,
    kDevNonFinite = 16u,
};

// ---------------------------------------------------------------------------
// Exact float32 squared distance in feature order, each operation rounded on
// its own (no fused multiply-add), as the oracle and the reference's x86-64
// build compute it.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float sq_term(float x, float c) {
    float t = __fsub_rn(x, c);
    return __fmul_rn(t, t);
}

// Eight floats of read-only data by one 256-bit load (p 32-byte aligned).
// A warp whose threads each walk their own row touches 32 cache lines per
// load instruction, and the L1 serves one line per cycle: 32-byte loads move
// twice the bytes of 16-byte ones per wavefront.
__device__ __forceinline__ void ldg_f32x8(const float *p, float (&v)[8]) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
        : "l"(p));
}

// 32 consecutive floats by four 256-bit loads issued together (one asm
// block, so that the compiler cannot spread them between the sums).
__device__ __forceinline__ void ldg_f32x32(const float *p, float (&v)[32]) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%32];\n\t"
        "ld.global.nc.v8.f32 {%8, %9, %10, %11, %12, %13, %14, %15}, [%32+32];\n\t"
        "ld.global.nc.v8.f32 {%16, %17, %18, %19, %20, %21, %22, %23}, [%32+64];\n\t"
        "ld.global.nc.v8.f32 {%24, %25, %26, %27, %28, %29, %30, %31}, [%32+96];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]),
          "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15]),
          "=f"(v[16]), "=f"(v[17]), "=f"(v[18]), "=f"(v[19]), "=f"(v[20]), "=f"(v[21]), "=f"(v[22]), "=f"(v[23]),
          "=f"(v[24]), "=f"(v[25]), "=f"(v[26]), "=f"(v[27]), "=f"(v[28]), "=f"(v[29]), "=f"(v[30]), "=f"(v[31])
        : "l"(p));
}

__device__ __forceinline__ float sqdist_exact(const float *__restrict__ x, const float *__restrict__ c,
                                              int d) {
    float acc = 0.0f;
    if ((d & 7) == 0 && ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(c)) & 31) == 0) {
        // Groups of four 32-byte loads per row are issued before their sums,
        // so a thread waits for memory once per 32 features, not per 8.
        int f = 0;
        for (; f + 32 <= d; f += 32) {
            float a[32], b[32];
            ldg_f32x32(x + f, a);
            ldg_f32x32(c + f, b);
#pragma unroll
            for (int q = 0; q < 32; ++q) acc = __fadd_rn(acc, sq_term(a[q], b[q]));
        }
        for (; f < d; f += 8) {
            float a[8], b[8];
            ldg_f32x8(x + f, a);
            ldg_f32x8(c + f, b);
#pragma unroll
            for (int q = 0; q < 8; ++q) acc = __fadd_rn(acc, sq_term(a[q], b[q]));
        }
    } else if ((d & 3) == 0 && ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(c)) & 15) == 0) {
        const float4 *x4 = reinterpret_cast<const float4 *>(x);
        const float4 *c4 = reinterpret_cast<const float4 *>(c);
        for (int f = 0; f < (d >> 2); ++f) {
            float4 a = __ldg(x4 + f);
            float4 b = __ldg(c4 + f);
            acc = __fadd_rn(acc, sq_term(a.x, b.x));
            acc = __fadd_rn(acc, sq_term(a.y, b.y));
            acc = __fadd_rn(acc, sq_term(a.z, b.z));
            acc = __fadd_rn(acc, sq_term(a.w, b.w));
        }
    } else {
        for (int f = 0; f < d; ++f) acc = __fadd_rn(acc, sq_term(__ldg(x + f), __ldg(c + f)));
    }
    return acc;
}

// ---------------------------------------------------------------------------
// Frame rows of the kernels that read float32 features: a dense row-major
// (n, d) matrix, or atom-pair distances computed from coordinates on the fly
// (the featurization fused into the discretization).  A pair feature is the
// float32 value km_pair_distances writes, bit for bit:
//   sqrt((dx*dx + dy*dy) + dz*dz),  (dx, dy, dz) = xyz[pair.y] - xyz[pair.x].
// ---------------------------------------------------------------------------
struct DenseRows {
    const float *X;
    int d;
    __device__ __forceinline__ float get(int64_t i, int f) const { return __ldg(X + i * d + f); }
};

// 4-byte asynchronous copies global -> shared (no alignment rule beyond 4
// bytes), committed in groups; cp_async_wait<N> returns once at most N of
// this thread's groups are still in flight.  Other lanes see the data after
// their own wait and a __syncwarp.
__device__ __forceinline__ void cp_async4(float *dst, const float *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// The distance of atoms a and b: one rounding per operation, in the order
// sqrt((dx^2 + dy^2) + dz^2) with d = b - a.  Every kernel that computes a
// pair feature goes through this function.
__device__ __forceinline__ float pair_feature(float ax, float ay, float az, float bx, float by, float bz) {
    const float dx = __fsub_rn(bx, ax);
    const float dy = __fsub_rn(by, ay);
    const float dz = __fsub_rn(bz, az);
    return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
}

struct PairRows {
    const float *xyz;   // (n, n_atoms, 3) frame-major
    const int2 *pairs;  // d atom pairs
    int n_atoms;
    int d;
    __device__ __forceinline__ float get(int64_t i, int f) const {
        const int2 p = __ldg(pairs + f);
        const float *a = xyz + (i * n_atoms + p.x) * 3;
        const float *b = xyz + (i * n_atoms + p.y) * 3;
        return pair_feature(__ldg(a), __ldg(a + 1), __ldg(a + 2), __ldg(b), __ldg(b + 1), __ldg(b + 2));
    }
};

// The exact float32 squared distance of sqdist_exact for a row source.
template <class Src>
__device__ __forceinline__ float sqdist_exact_src(const Src &src, int64_t i, const float *__restrict__ c, int d) {
    float acc = 0.0f;
    for (int f = 0; f < d; ++f) acc = __fadd_rn(acc, sq_term(src.get(i, f), __ldg(c + f)));
    return acc;
}

// Neumaier-compensated float32 sum: value() is within a few u of the exact
// sum of the added terms (plus an O(n u^2) remainder).
struct CSum {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float v) {
        const float t = s + v;
        c += fabsf(s) >= fabsf(v) ? (s - t) + v : (v - t) + s;
        s = t;
    }
    __device__ __forceinline__ void reset() {
        s = 0.0f;
        c = 0.0f;
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// Lexicographic (distance, index) minimum across a warp; NaN never wins.
__device__ __forceinline__ void warp_argmin(float &bd, int &bj) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        float od = __shfl_xor_sync(0xffffffffu, bd, off);
        int oj = __shfl_xor_sync(0xffffffffu, bj, off);
        if (od < bd || (od == bd && oj < bj)) {
            bd = od;
            bj = oj;
        }
    }
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11) and the kmeans++ draw of round r.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = uint64_t(0xD2511F53u) * c[0];
        uint64_t p1 = uint64_t(0xCD9E8D57u) * c[2];
        uint32_t n0 = uint32_t(p1 >> 32) ^ c[1] ^ k0;
        uint32_t n2 = uint32_t(p0 >> 32) ^ c[3] ^ k1;
        c[1] = uint32_t(p1);
        c[3] = uint32_t(p0);
        c[0] = n0;
        c[2] = n2;
    }
}

__host__ __device__ __forceinline__ uint64_t kmpp_draw(uint32_t seed, uint32_t round) {
    uint32_t c[4] = {round, 0u, 0x6B6D7070u, 0u};
    philox4x32_10(c, seed, 0x4B4D4750u);
    return (uint64_t(c[0]) << 32) | uint64_t(c[1]);
}

// ---------------------------------------------------------------------------
// Bounded waits: a spin gives up after kWaitLimitNs of wall time.
// ---------------------------------------------------------------------------
constexpr uint64_t kWaitLimitNs = 4000000000ull;  // 4 s

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

}  // namespace km

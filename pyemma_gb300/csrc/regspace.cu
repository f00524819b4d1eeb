// regspace.cu -- regular space clustering, first pass (km_regspace).
//
// Reference: RegularSpaceClustering._estimate, pyemma/coordinates/clustering/
// regspace.py:140-152 (deeptime RegularSpace.partial_fit over the chunks in
// iteration order).  The first frame becomes a center; every later frame
// becomes one when its distance to every center found so far is at least
// dmin.  The distance is the square root (float32, correctly rounded) of the
// exact float32 squared distance in feature order, compared in double with
// dmin.
//
// The walk is sequential by definition; the GPU splits it by chunks of
// frames.  For a chunk, the exact FP32 assignment kernel gives every frame's
// smallest squared distance to the centers known before the chunk.  One CTA
// then walks the chunk in frame order, 256 frames at a time: the frames that
// pass against the earlier centers are compacted in order, and each of them
// is tested against the centers added within the chunk (one thread per
// center) and appended when it passes.
#include "km_common.cuh"
#include "km_internal.h"

namespace km {

namespace {

constexpr int64_t kRsChunk = 65536;
constexpr int kRsThreads = 256;

// sqdist_exact's arithmetic and order, with the center rows read around the
// non-coherent read-only cache: they are appended by this same kernel.
__device__ __forceinline__ float sqdist_to_new_center(const float *__restrict__ x, const float *c, int d) {
    float acc = 0.0f;
    for (int f = 0; f < d; ++f) acc = __fadd_rn(acc, sq_term(__ldg(x + f), __ldcg(c + f)));
    return acc;
}

__global__ void __launch_bounds__(kRsThreads) regspace_walk_kernel(
    const float *__restrict__ X, int64_t a, int64_t b, int d, const float *__restrict__ dist2, double dmin,
    int max_centers, float *__restrict__ centers, int32_t *__restrict__ state) {
    __shared__ int cand[kRsThreads];
    __shared__ int ncand;
    __shared__ int s_nc;
    __shared__ int s_stop;
    const int tid = threadIdx.x;
    const int nc0 = state[0];
    if (tid == 0) {
        s_nc = nc0;
        s_stop = 0;
    }
    __syncthreads();
    for (int64_t base = a; base < b; base += kRsThreads) {
        // Frames of this batch that pass against the centers before the chunk,
        // in frame order.
        const int64_t i = base + tid;
        bool pass = false;
        if (i < b) pass = dist2 == nullptr || (double)__fsqrt_rn(dist2[i - a]) >= dmin;
        if (tid == 0) ncand = 0;
        __syncthreads();
        const unsigned ballot = __ballot_sync(0xffffffffu, pass);
        __shared__ int warp_count[kRsThreads / 32];
        if ((tid & 31) == 0) warp_count[tid >> 5] = __popc(ballot);
        __syncthreads();
        if (pass) {
            int pos = __popc(ballot & ((1u << (tid & 31)) - 1u));
            for (int w = 0; w < (tid >> 5); ++w) pos += warp_count[w];
            cand[pos] = (int)(i - a);
        }
        if (tid == 0) {
            int t = 0;
            for (int w = 0; w < kRsThreads / 32; ++w) t += warp_count[w];
            ncand = t;
        }
        __syncthreads();
        const int nb = ncand;
        for (int q = 0; q < nb; ++q) {
            const int64_t f = a + cand[q];
            const float *x = X + f * d;
            const int nc = s_nc;
            // Against the centers added within this chunk.
            bool fail = false;
            for (int j = nc0 + tid; j < nc; j += kRsThreads) {
                const float dd = __fsqrt_rn(sqdist_to_new_center(x, centers + (int64_t)j * d, d));
                if (!((double)dd >= dmin)) fail = true;
            }
            const int any_fail = __syncthreads_or(fail);
            if (!any_fail) {
                if (nc == max_centers) {
                    if (tid == 0) s_stop = 1;
                } else {
                    for (int c = tid; c < d; c += kRsThreads) centers[(int64_t)nc * d + c] = x[c];
                    __threadfence_block();
                    if (tid == 0) s_nc = nc + 1;
                }
            }
            __syncthreads();
            if (s_stop) break;
        }
        if (s_stop) break;
    }
    __syncthreads();
    if (tid == 0) {
        state[0] = s_nc;
        state[1] = s_stop;
    }
}

}  // namespace

}  // namespace km

using namespace km;

extern "C" {

size_t km_regspace_workspace_size(int32_t d) {
    if (d < 1 || d > kMaxD) return 0;
    Carver c(nullptr);
    c.take<int32_t>(kRsChunk);
    c.take<float>(kRsChunk);
    c.take<int32_t>(2);
    return c.bytes();
}

int km_regspace(const float *X, int64_t n, int32_t d, double dmin, int32_t max_centers, float *centers,
                int32_t *n_centers, int32_t *converged, void *workspace, size_t workspace_bytes, void *stream) {
    if (!n_centers || !converged) {
        set_error("n_centers and converged must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    *n_centers = 0;
    *converged = 1;
    KM_TRY(check_shape(n, d, max_centers > 0 ? max_centers : 1));
    if (max_centers < 1 || !(dmin >= 0.0) || (n > 0 && (!X || !centers))) {
        set_error("km_regspace needs max_centers >= 1, dmin >= 0 and non-NULL X, centers");
        return KM_ERR_BAD_SHAPE;
    }
    KM_TRY(check_ws(workspace, workspace_bytes, km_regspace_workspace_size(d)));
    if (n == 0) return KM_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Carver cv(workspace);
    int32_t *labels = cv.take<int32_t>(kRsChunk);
    float *dist = cv.take<float>(kRsChunk);
    int32_t *state = cv.take<int32_t>(2);
    KM_CUDA(cudaMemsetAsync(state, 0, 2 * sizeof(int32_t), s));
    int32_t h_state[2] = {0, 0};
    for (int64_t a = 0; a < n; a += kRsChunk) {
        const int64_t b = a + kRsChunk < n ? a + kRsChunk : n;
        if (h_state[0] > 0)
            KM_TRY(launch_assign_fp32(X + a * d, nullptr, nullptr, b - a, d, centers, h_state[0], labels, dist,
                                      nullptr, s));
        regspace_walk_kernel<<<1, kRsThreads, 0, s>>>(X, a, b, d, h_state[0] > 0 ? dist : nullptr, dmin,
                                                      max_centers, centers, state);
        KM_CUDA(cudaGetLastError());
        KM_CUDA(cudaMemcpyAsync(h_state, state, sizeof(h_state), cudaMemcpyDeviceToHost, s));
        KM_CUDA(cudaStreamSynchronize(s));
        if (h_state[1]) break;
    }
    *n_centers = h_state[0];
    *converged = h_state[1] ? 0 : 1;
    return KM_OK;
}

}  // extern "C"

// counts.cu -- lag-tau transition counts of discrete trajectories
// (km_count_matrix).
//
// Reference: the step after discretization, pyemma/msm/estimators/
// _dtraj_stats.py:139-145 (count_matrix(dtrajs, lag, sliding) and
// TransitionCountEstimator of deeptime): for every trajectory the pairs
// (dtraj[t], dtraj[t + lag]) for t = 0, 1, ..., T - lag - 1 (sliding) or
// t = 0, lag, 2 lag, ... < T - lag (sample) are counted into a dense
// nstates x nstates matrix; pairs with a negative state (unassigned frames)
// are left out.
//
// One thread per time index of the packed trajectories; the trajectory of
// an index is found by binary search over the offsets.  Threads of a warp
// that hold the same (from, to) pair are merged with __match_any_sync, so the
// long self-transition runs of metastable trajectories cost one atomic per
// warp instead of one per frame.
#include "km_common.cuh"
#include "km_internal.h"

namespace km {

namespace {

__global__ void __launch_bounds__(256) count_pairs_kernel(const int32_t *__restrict__ dtrajs,
                                                          const int64_t *__restrict__ offsets, int n_traj,
                                                          int64_t n, int lag, int sliding, int nstates,
                                                          unsigned long long *__restrict__ counts) {
    const int lane = threadIdx.x & 31;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = base + threadIdx.x;
        long long key = -1;
        if (p < n) {
            // trajectory of position p: the last t with offsets[t] <= p
            int lo = 0, hi = n_traj - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (offsets[mid] <= p)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            const int64_t t = p - offsets[lo];
            const int64_t T = offsets[lo + 1] - offsets[lo];
            const bool take = t + lag < T && (sliding || t % lag == 0);
            if (take) {
                const int a = dtrajs[p];
                const int b = dtrajs[p + lag];
                if (a >= 0 && b >= 0 && a < nstates && b < nstates) key = (long long)a * nstates + b;
            }
        }
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        if (key >= 0 && lane == __ffs(peers) - 1) atomicAdd(&counts[key], (unsigned long long)__popc(peers));
    }
}

}  // namespace

}  // namespace km

using namespace km;

extern "C" {

size_t km_count_matrix_workspace_size(int32_t n_traj) {
    if (n_traj < 0) return 0;
    Carver c(nullptr);
    c.take<int64_t>((size_t)n_traj + 1);
    return c.bytes();
}

int km_count_matrix(const int32_t *dtrajs, const int64_t *offsets, int32_t n_traj, int32_t lag, int32_t sliding,
                    int32_t nstates, int64_t *counts, void *workspace, size_t workspace_bytes, void *stream) {
    if (n_traj < 0 || (n_traj > 0 && !offsets) || lag < 1 || nstates < 1 || !counts) {
        set_error("km_count_matrix needs n_traj >= 0 with offsets, lag >= 1, nstates >= 1 and counts");
        return KM_ERR_BAD_SHAPE;
    }
    if ((int64_t)nstates * nstates > (int64_t(1) << 31)) {
        set_error("nstates=%d: the dense count matrix would exceed 2^31 entries", nstates);
        return KM_ERR_BAD_SHAPE;
    }
    if (n_traj > 0 && offsets[0] != 0) {
        set_error("offsets[0] must be 0");
        return KM_ERR_BAD_SHAPE;
    }
    for (int32_t t = 0; t < n_traj; ++t) {
        if (offsets[t + 1] < offsets[t]) {
            set_error("offsets must be non-decreasing (trajectory %d)", t);
            return KM_ERR_BAD_SHAPE;
        }
    }
    KM_TRY(check_ws(workspace, workspace_bytes, km_count_matrix_workspace_size(n_traj)));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    KM_CUDA(cudaMemsetAsync(counts, 0, sizeof(int64_t) * (size_t)nstates * nstates, s));
    const int64_t n = n_traj > 0 ? offsets[n_traj] : 0;
    if (n == 0) return KM_OK;
    if (!dtrajs) {
        set_error("dtrajs must be non-NULL");
        return KM_ERR_BAD_SHAPE;
    }
    int64_t *d_offsets = static_cast<int64_t *>(workspace);
    KM_CUDA(cudaMemcpyAsync(d_offsets, offsets, sizeof(int64_t) * ((size_t)n_traj + 1), cudaMemcpyHostToDevice, s));
    int64_t g = (n + 255) / 256;
    const int64_t cap = (int64_t)num_sms() * 8;
    if (g > cap) g = cap;
    count_pairs_kernel<<<(unsigned)g, 256, 0, s>>>(dtrajs, d_offsets, n_traj, n, lag, sliding ? 1 : 0, nstates,
                                                   reinterpret_cast<unsigned long long *>(counts));
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

}  // extern "C"

// featurize.cu -- atom-pair distance features on the device
// (km_pair_distances).
//
// Reference: the featurization feeding the discretization,
// pyemma/coordinates/data/featurization/featurizer.py:305-372
// (add_distances / add_distances_ca) and distances.py:53-54
// (mdtraj.compute_distances without a unit cell): feature p of frame t is
// the Euclidean distance between atoms pairs[p].x and pairs[p].y.  In float32
// with every operation rounded on its own:
//   sqrt((dx*dx + dy*dy) + dz*dz),  d = xyz[j] - xyz[i].
// Computing the features on the device from the (T, n_atoms, 3) coordinates
// moves n_atoms * 12 bytes per frame to the GPU instead of 4 * n_pairs
// (396 vs 2,112 bytes for a 33-bead chain with all pairs).
//
// One thread per output feature in frame-major order, so the writes of a
// warp are coalesced; the coordinates of the frame come through L1.
#include <vector>

#include "km_common.cuh"
#include "km_internal.h"

namespace km {

namespace {

// A warp per frame (frames in a grid-stride walk), lanes over the pairs:
// coalesced writes, the frame's coordinates from L1 after their first read,
// and no 64-bit division per feature.
__global__ void __launch_bounds__(256) pair_distances_kernel(const float *__restrict__ xyz, int64_t n, int n_atoms,
                                                             const int2 *__restrict__ pairs, int npairs,
                                                             float *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t t = w; t < n; t += nw) {
        const float *x = xyz + t * n_atoms * 3;
        float *o = out + t * npairs;
        for (int p = lane; p < npairs; p += 32) {
            const int2 ij = __ldg(pairs + p);
            const float *a = x + ij.x * 3;
            const float *b = x + ij.y * 3;
            o[p] = pair_feature(__ldg(a), __ldg(a + 1), __ldg(a + 2), __ldg(b), __ldg(b + 1), __ldg(b + 2));
        }
    }
}

}  // namespace

// Atom pairs (device, npairs x 2) are read back (a few KB) and checked on the
// host: an index outside [0, n_atoms) would make every kernel that computes
// the features read outside the coordinates.
int check_pairs(const int32_t *pairs, int32_t npairs, int32_t n_atoms, cudaStream_t s) {
    if (npairs <= 0) return KM_OK;
    std::vector<int32_t> h((size_t)npairs * 2);
    KM_CUDA(cudaMemcpyAsync(h.data(), pairs, h.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    KM_CUDA(cudaStreamSynchronize(s));
    for (size_t q = 0; q < h.size(); ++q)
        if (h[q] < 0 || h[q] >= n_atoms) {
            set_error("pair %zu names atom %d, outside [0, %d)", q / 2, h[q], n_atoms);
            return KM_ERR_BAD_SHAPE;
        }
    return KM_OK;
}

}  // namespace km

using namespace km;

extern "C" {

int km_pair_distances(const float *xyz, int64_t n, int32_t n_atoms, const int32_t *pairs, int32_t npairs,
                      float *out, void *stream) {
    if (n < 0 || n_atoms < 1 || npairs < 0 || (n > 0 && npairs > 0 && (!xyz || !pairs || !out))) {
        set_error("km_pair_distances needs n >= 0, n_atoms >= 1, npairs >= 0 and non-NULL arrays");
        return KM_ERR_BAD_SHAPE;
    }
    const int64_t total = n * (int64_t)npairs;
    if (total == 0) return KM_OK;
    KM_TRY(check_pairs(pairs, npairs, n_atoms, static_cast<cudaStream_t>(stream)));
    int64_t g = (n * 32 + 255) / 256;  // a warp per frame
    const int64_t cap = (int64_t)num_sms() * 16;
    if (g > cap) g = cap;
    pair_distances_kernel<<<(unsigned)g, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        xyz, n, n_atoms, reinterpret_cast<const int2 *>(pairs), npairs, out);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

}  // extern "C"

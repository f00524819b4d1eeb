// minrmsd.cu -- k-means under the minRMSD metric: assignment, the metric of
// row pairs, kmeans++ and Lloyd iterations (km_*_minrmsd).
//
// Reference: the minRMSD metric plug-in, pyemma/coordinates/clustering/src/
// clustering_module.cpp:9-36, registered into deeptime's clustering and
// reached through cluster_kmeans(metric='minRMSD') / assign_to_centers(
// metric='minRMSD') (pyemma/coordinates/api.py, clustering/kmeans.py:114-115).
// Frames are atom-major rows of d = 3 n_atoms floats.  The squared metric is
// the mean square deviation after optimal superposition (km_rmsd.cuh); the
// label is the lowest index with the smallest msd.  The center update of a
// Lloyd iteration is the mean of the members, as for the Euclidean metric;
// the inertia is the sum of the members' msd to their new centers.
//
// Layout: frames and centers are centered once into float copies with their
// traces G (double).  The centered centers are also stored transposed
// (feature-major, k padded to 32) so that the lanes of a warp, one center
// each, read them coalesced.  The assignment kernel gives one warp to one
// frame: the frame's coordinates are the same for every lane (broadcast
// loads), each lane accumulates the nine correlation sums of its center in
// atom order, solves the QCP quartic in double, and the warp keeps the
// lowest-index minimum.
#include "km_common.cuh"
#include "km_internal.h"
#include "km_rmsd.cuh"

namespace km {

namespace {

constexpr int kRmsdWarps = 8;  // warps per CTA

// Every row of an (n, d) array centered into Xc, traces into G.
__global__ void __launch_bounds__(kRmsdWarps * 32) rmsd_center_kernel(const float *__restrict__ X, int64_t n, int d,
                                                                      float *__restrict__ Xc, double *__restrict__ G) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * kRmsdWarps;
    for (int64_t r = (int64_t)blockIdx.x * kRmsdWarps + (threadIdx.x >> 5); r < n; r += nw) {
        const double g = rmsd_center_row_warp(X + r * d, d / 3, Xc + r * d);
        if (lane == 0) G[r] = g;
    }
}

// Ct[f * kp + j] = Cc[j * d + f]; zero for the padding centers.
__global__ void rmsd_transpose_kernel(const float *__restrict__ Cc, int k, int kp, int d, float *__restrict__ Ct) {
    const int64_t total = (int64_t)kp * d;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int f = (int)(e / kp), j = (int)(e - (int64_t)f * kp);
        Ct[e] = j < k ? Cc[(int64_t)j * d + f] : 0.0f;
    }
}

// (msd, index) of the better of two candidates: a number beats NaN or no
// candidate (index < 0), then the smaller msd, then the lower index.
__device__ __forceinline__ bool rmsd_better(double m, int j, double bm, int bj) {
    if (j < 0 || m != m) return false;
    if (bj < 0) return true;
    return m < bm || (m == bm && j < bj);
}

__global__ void __launch_bounds__(kRmsdWarps * 32) rmsd_assign_kernel(
    const float *__restrict__ Xc, const double *__restrict__ G, int64_t n, int d, const float *__restrict__ Ct,
    const double *__restrict__ H, int k, int kp, int32_t *__restrict__ labels, float *__restrict__ rmsd) {
    const int lane = threadIdx.x & 31;
    const int n_atoms = d / 3;
    const int64_t nw = (int64_t)gridDim.x * kRmsdWarps;
    for (int64_t r = (int64_t)blockIdx.x * kRmsdWarps + (threadIdx.x >> 5); r < n; r += nw) {
        const float *a = Xc + r * d;
        const double ga = G[r];
        double bm = 0.0;
        int bj = -1;
        for (int j0 = 0; j0 < k; j0 += 32) {
            const int j = j0 + lane;  // j < kp: the padding centers are zero rows
            float S[9];
#pragma unroll
            for (int e = 0; e < 9; ++e) S[e] = 0.0f;
            const float *b = Ct + j;
            for (int i = 0; i < n_atoms; ++i) {
                const float a0 = a[3 * i], a1 = a[3 * i + 1], a2 = a[3 * i + 2];
                const float b0 = b[(int64_t)(3 * i) * kp], b1 = b[(int64_t)(3 * i + 1) * kp],
                            b2 = b[(int64_t)(3 * i + 2) * kp];
                S[0] = __fmaf_rn(a0, b0, S[0]);
                S[1] = __fmaf_rn(a0, b1, S[1]);
                S[2] = __fmaf_rn(a0, b2, S[2]);
                S[3] = __fmaf_rn(a1, b0, S[3]);
                S[4] = __fmaf_rn(a1, b1, S[4]);
                S[5] = __fmaf_rn(a1, b2, S[5]);
                S[6] = __fmaf_rn(a2, b0, S[6]);
                S[7] = __fmaf_rn(a2, b1, S[7]);
                S[8] = __fmaf_rn(a2, b2, S[8]);
            }
            if (j < k) {
                const double m = qcp_msd(S, ga, H[j], n_atoms);
                if (rmsd_better(m, j, bm, bj)) {
                    bm = m;
                    bj = j;
                }
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const double om = __shfl_xor_sync(0xffffffffu, bm, off);
            const int oj = __shfl_xor_sync(0xffffffffu, bj, off);
            if (rmsd_better(om, oj, bm, bj)) {
                bm = om;
                bj = oj;
            }
        }
        if (lane == 0) {
            labels[r] = bj < 0 ? 0 : bj;
            if (rmsd) rmsd[r] = bj < 0 ? __int_as_float(0x7fc00000) : __double2float_rn(sqrt(bm));
        }
    }
}

// rmsd[i] = sqrt(msd(A[i], B[i])) of centered row pairs.
__global__ void rmsd_rows_kernel(const float *__restrict__ A, const double *__restrict__ GA,
                                 const float *__restrict__ B, const double *__restrict__ GB, int64_t n, int d,
                                 float *__restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = __double2float_rn(sqrt(rmsd_msd_rows(A + i * d, B + i * d, GA[i], GB[i], d / 3)));
}

// cost += sum_i msd(frame i, center labels[i]).
__global__ void __launch_bounds__(256) rmsd_cost_kernel(const float *__restrict__ Xc, const double *__restrict__ G,
                                                        int64_t n, int d, const int32_t *__restrict__ labels,
                                                        const float *__restrict__ Cc, const double *__restrict__ H,
                                                        double *__restrict__ cost) {
    __shared__ double red[8];
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int j = labels[i];
        s += rmsd_msd_rows(Xc + i * d, Cc + (int64_t)j * d, G[i], H[j], d / 3);
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += red[w];
        atomicAdd(cost, t);
    }
}

unsigned rmsd_grid(int64_t warps_needed) {
    int64_t g = (warps_needed + kRmsdWarps - 1) / kRmsdWarps;
    const int64_t cap = (int64_t)num_sms() * 8;
    if (g > cap) g = cap;
    return (unsigned)(g < 1 ? 1 : g);
}

int kp_of_k(int k) { return (k + 31) / 32 * 32; }

struct RmsdCenters {
    float *Cc;
    double *H;
    float *Ct;
};

RmsdCenters carve_centers(Carver &c, int d, int k) {
    RmsdCenters r;
    r.Cc = c.take<float>((size_t)k * d);
    r.H = c.take<double>((size_t)k);
    r.Ct = c.take<float>((size_t)kp_of_k(k) * d);
    return r;
}

int check_rmsd_shape(int64_t n, int d, int k) {
    KM_TRY(check_shape(n, d, k));
    if (d % 3 != 0) {
        set_error("the minRMSD metric needs atom-major rows of 3 n_atoms floats (d=%d is not divisible by 3)", d);
        return KM_ERR_BAD_SHAPE;
    }
    return KM_OK;
}

int center_rows(const float *X, int64_t n, int d, float *Xc, double *G, cudaStream_t s) {
    if (n == 0) return KM_OK;
    rmsd_center_kernel<<<rmsd_grid(n), kRmsdWarps * 32, 0, s>>>(X, n, d, Xc, G);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

int prepare_centers(const float *C, int d, int k, const RmsdCenters &rc, cudaStream_t s) {
    KM_TRY(center_rows(C, k, d, rc.Cc, rc.H, s));
    const int kp = kp_of_k(k);
    int64_t g = ((int64_t)kp * d + 255) / 256;
    const int64_t cap = (int64_t)num_sms() * 8;
    if (g > cap) g = cap;
    rmsd_transpose_kernel<<<(unsigned)(g < 1 ? 1 : g), 256, 0, s>>>(rc.Cc, k, kp, d, rc.Ct);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

int launch_rmsd_assign(const float *Xc, const double *G, int64_t n, int d, const RmsdCenters &rc, int k,
                       int32_t *labels, float *rmsd, cudaStream_t s) {
    if (n == 0) return KM_OK;
    rmsd_assign_kernel<<<rmsd_grid(n), kRmsdWarps * 32, 0, s>>>(Xc, G, n, d, rc.Ct, rc.H, k, kp_of_k(k), labels,
                                                               rmsd);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

}  // namespace

}  // namespace km

using namespace km;

extern "C" {

size_t km_assign_minrmsd_workspace_size(int64_t n, int32_t d, int32_t k) {
    if (check_rmsd_shape(n, d, k) != KM_OK) return 0;
    Carver c(nullptr);
    c.take<float>((size_t)(n > 0 ? n : 1) * d);
    c.take<double>((size_t)(n > 0 ? n : 1));
    carve_centers(c, d, k);
    return c.bytes();
}

int km_assign_minrmsd(const float *X, int64_t n, int32_t d, const float *C, int32_t k, int32_t *labels, float *rmsd,
                      void *workspace, size_t workspace_bytes, void *stream) {
    KM_TRY(check_rmsd_shape(n, d, k));
    if ((n > 0 && (!X || !labels)) || !C) {
        set_error("km_assign_minrmsd needs non-NULL X, C and labels");
        return KM_ERR_BAD_SHAPE;
    }
    KM_TRY(check_ws(workspace, workspace_bytes, km_assign_minrmsd_workspace_size(n, d, k)));
    if (n == 0) return KM_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Carver c(workspace);
    float *Xc = c.take<float>((size_t)n * d);
    double *G = c.take<double>((size_t)n);
    RmsdCenters rc = carve_centers(c, d, k);
    KM_TRY(center_rows(X, n, d, Xc, G, s));
    KM_TRY(prepare_centers(C, d, k, rc, s));
    return launch_rmsd_assign(Xc, G, n, d, rc, k, labels, rmsd, s);
}

size_t km_minrmsd_rows_workspace_size(int64_t n, int32_t d) {
    if (check_rmsd_shape(n, d, 1) != KM_OK) return 0;
    Carver c(nullptr);
    for (int t = 0; t < 2; ++t) {
        c.take<float>((size_t)(n > 0 ? n : 1) * d);
        c.take<double>((size_t)(n > 0 ? n : 1));
    }
    return c.bytes();
}

int km_minrmsd_rows(const float *X, const float *Y, int64_t n, int32_t d, float *rmsd, void *workspace,
                    size_t workspace_bytes, void *stream) {
    KM_TRY(check_rmsd_shape(n, d, 1));
    if (n > 0 && (!X || !Y || !rmsd)) {
        set_error("km_minrmsd_rows needs non-NULL X, Y and rmsd");
        return KM_ERR_BAD_SHAPE;
    }
    KM_TRY(check_ws(workspace, workspace_bytes, km_minrmsd_rows_workspace_size(n, d)));
    if (n == 0) return KM_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Carver c(workspace);
    float *A = c.take<float>((size_t)n * d);
    double *GA = c.take<double>((size_t)n);
    float *B = c.take<float>((size_t)n * d);
    double *GB = c.take<double>((size_t)n);
    KM_TRY(center_rows(X, n, d, A, GA, s));
    KM_TRY(center_rows(Y, n, d, B, GB, s));
    int64_t g = (n + 255) / 256;
    const int64_t cap = (int64_t)num_sms() * 8;
    if (g > cap) g = cap;
    rmsd_rows_kernel<<<(unsigned)g, 256, 0, s>>>(A, GA, B, GB, n, d, rmsd);
    KM_CUDA(cudaGetLastError());
    return KM_OK;
}

size_t km_kmpp_minrmsd_workspace_size(int64_t n, int32_t d, int32_t k) {
    if (check_rmsd_shape(n, d, k) != KM_OK) return 0;
    Carver c(nullptr);
    c.take<float>((size_t)(n > 0 ? n : 1) * d);
    c.take<double>((size_t)(n > 0 ? n : 1));
    c.take<int64_t>((size_t)k);
    c.take<char>(kmpp_ws_size(n, d, k));
    return c.bytes();
}

int km_kmpp_minrmsd(const float *X, int64_t n, int32_t d, int32_t k, uint32_t seed, float *C0, int64_t *idx,
                    km_callback cb, void *cb_user, void *workspace, size_t workspace_bytes, void *stream) {
    KM_TRY(check_rmsd_shape(n, d, k));
    if (n < 1 || !X || !C0) {
        set_error("kmeans++ needs n >= 1 and non-NULL X, C0");
        return KM_ERR_BAD_SHAPE;
    }
    KM_TRY(check_ws(workspace, workspace_bytes, km_kmpp_minrmsd_workspace_size(n, d, k)));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Carver c(workspace);
    float *Xc = c.take<float>((size_t)n * d);
    double *G = c.take<double>((size_t)n);
    int64_t *idx_dev = c.take<int64_t>((size_t)k);
    void *ws_kmpp = c.take<char>(kmpp_ws_size(n, d, k));
    KM_TRY(center_rows(X, n, d, Xc, G, s));
    KmppMetric m{Xc, G, idx_dev};
    KM_TRY(run_kmpp(X, n, d, k, seed, C0, idx_dev, cb, cb_user, ws_kmpp, s, &m));
    if (idx) KM_CUDA(cudaMemcpyAsync(idx, idx_dev, sizeof(int64_t) * (size_t)k, cudaMemcpyDeviceToDevice, s));
    return KM_OK;
}

size_t km_lloyd_minrmsd_workspace_size(int64_t n, int32_t d, int32_t k) {
    if (check_rmsd_shape(n, d, k) != KM_OK) return 0;
    Carver c(nullptr);
    c.take<float>((size_t)(n > 0 ? n : 1) * d);
    c.take<double>((size_t)(n > 0 ? n : 1));
    carve_centers(c, d, k);
    c.take<float>((size_t)k * d);  // C_new
    c.take<double>(2);             // cost, the update's own cost
    c.take<uint32_t>(1);
    c.take<char>(update_ws_size(n, d, k));
    return c.bytes();
}

int km_lloyd_minrmsd(const float *X, int64_t n, int32_t d, int32_t k, float *C, int32_t max_iter, double tolerance,
                     int32_t *labels, double *inertias, int32_t *n_iter, int32_t *converged, km_callback cb,
                     void *cb_user, void *workspace, size_t workspace_bytes, void *stream) {
    KM_TRY(check_rmsd_shape(n, d, k));
    if (n < 1 || !X || !C || !labels || !n_iter || !converged || max_iter < 0) {
        set_error("km_lloyd_minrmsd needs n >= 1, max_iter >= 0 and non-NULL X, C, labels, n_iter, converged");
        return KM_ERR_BAD_SHAPE;
    }
    *n_iter = 0;
    *converged = 0;
    KM_TRY(check_ws(workspace, workspace_bytes, km_lloyd_minrmsd_workspace_size(n, d, k)));
    if (max_iter == 0) return KM_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Carver c(workspace);
    float *Xc = c.take<float>((size_t)n * d);
    double *G = c.take<double>((size_t)n);
    RmsdCenters rc = carve_centers(c, d, k);
    float *C_new = c.take<float>((size_t)k * d);
    double *cost = c.take<double>(2);
    uint32_t *err = c.take<uint32_t>(1);
    void *ws_update = c.take<char>(update_ws_size(n, d, k));
    KM_TRY(center_rows(X, n, d, Xc, G, s));
    KM_CUDA(cudaMemsetAsync(err, 0, sizeof(uint32_t), s));
    double prev = 0.0;
    for (int32_t it = 0; it < max_iter; ++it) {
        KM_TRY(prepare_centers(C, d, k, rc, s));
        KM_TRY(launch_rmsd_assign(Xc, G, n, d, rc, k, labels, nullptr, s));
        KM_TRY(launch_update(X, n, d, labels, k, C, C_new, nullptr, cost + 1, err, ws_update, s));
        // inertia under the metric, for the new centers
        KM_TRY(center_rows(C_new, k, d, rc.Cc, rc.H, s));
        KM_CUDA(cudaMemsetAsync(cost, 0, sizeof(double), s));
        int64_t g = (n + 255) / 256;
        const int64_t cap = (int64_t)num_sms() * 8;
        if (g > cap) g = cap;
        rmsd_cost_kernel<<<(unsigned)g, 256, 0, s>>>(Xc, G, n, d, labels, rc.Cc, rc.H, cost);
        KM_CUDA(cudaGetLastError());
        KM_CUDA(cudaMemcpyAsync(C, C_new, sizeof(float) * (size_t)k * d, cudaMemcpyDeviceToDevice, s));
        double h_cost = 0.0;
        uint32_t h_err = 0;
        KM_CUDA(cudaMemcpyAsync(&h_cost, cost, sizeof(double), cudaMemcpyDeviceToHost, s));
        KM_CUDA(cudaMemcpyAsync(&h_err, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        KM_CUDA(cudaStreamSynchronize(s));
        KM_TRY(device_error_status(h_err));
        if (inertias) inertias[it] = h_cost;
        *n_iter = it + 1;
        const double rel = h_cost != 0.0 ? fabs(h_cost - prev) / h_cost : 0.0;
        prev = h_cost;
        if (cb) cb(cb_user);
        if (rel <= tolerance) {
            *converged = 1;
            break;
        }
    }
    return KM_OK;
}

}  // extern "C"

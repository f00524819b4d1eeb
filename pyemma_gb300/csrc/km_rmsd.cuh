// km_rmsd.cuh -- the minRMSD metric on the device: centering of atom-major
// rows and the quaternion characteristic polynomial (QCP) mean square
// deviation of two centered rows.
//
// Reference: the minRMSD metric of pyemma/coordinates/clustering/src/
// clustering_module.cpp:9-36 (RMSDMetric::compute_squared: both rows
// centered, then mdtraj's msd_atom_major, Theobald's QCP method, Acta Cryst.
// A61:478-480, 2005).  The arithmetic below fixes one order of operations,
// which the CPU oracle restates operation for operation, so that labels are
// equal bit for bit:
//   * centering: per axis a double sum over atoms in a 32-lane order (lane l
//     sums atoms l, l+32, ...; then an xor butterfly), mean = sum / n_atoms,
//     a = (float)(x - mean); G = sum a^2 in double in the same lane order;
//   * S[p][q] = sum_i a_i[p] b_i[q] as float fused multiply-adds in atom
//     order;
//   * in double, without contraction: C2 = -2 sum S^2, C1 = -8 det S,
//     C0 = det K, Newton on the quartic P from the smaller of two upper
//     bounds of its largest root, (Ga + Gb) / 2 and sqrt(3) ||S||_F =
//     sqrt(-1.5 C2) (float root, inflated by 1e-6; the largest eigenvalue of
//     the key matrix is at most the sum of the singular values of S), at most
//     50 steps until |step| < 1e-11 |lambda|, msd = max(0, (Ga + Gb -
//     2 lambda) / n).  P and P' are evaluated in double; the step is P times
//     the float reciprocal of (float)P' (P / P' when that is outside float's
//     range).  The root is P's, and the derivative
//     only scales the step: this keeps the double divisions off the FP64
//     pipe, which runs at a small fraction of the FP32 rate here.
#pragma once

#include <cstdint>

namespace km {

// Sum over the 32 lanes of a warp in xor-butterfly order (every lane gets the
// same value).
__device__ __forceinline__ double warp_butterfly_d(double s) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s = __dadd_rn(s, __shfl_xor_sync(0xffffffffu, s, off));
    return s;
}

// One warp centers one atom-major row x (n_atoms atoms) into a; returns G in
// every lane.
__device__ __forceinline__ double rmsd_center_row_warp(const float *__restrict__ x, int n_atoms,
                                                       float *__restrict__ a) {
    const int lane = threadIdx.x & 31;
    double mean[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        double acc = 0.0;
        for (int i = lane; i < n_atoms; i += 32) acc = __dadd_rn(acc, (double)x[3 * i + c]);
        mean[c] = __ddiv_rn(warp_butterfly_d(acc), (double)n_atoms);
    }
    double g = 0.0;
    for (int i = lane; i < n_atoms; i += 32) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float v = __double2float_rn(__dsub_rn((double)x[3 * i + c], mean[c]));
            a[3 * i + c] = v;
            g = __dadd_rn(g, __dmul_rn((double)v, (double)v));
        }
    }
    return warp_butterfly_d(g);
}

__device__ __forceinline__ double det3_d(double a, double b, double c, double d, double e, double f, double g,
                                         double h, double i) {
    const double t1 = __dmul_rn(a, __dsub_rn(__dmul_rn(e, i), __dmul_rn(f, h)));
    const double t2 = __dmul_rn(b, __dsub_rn(__dmul_rn(d, i), __dmul_rn(f, g)));
    const double t3 = __dmul_rn(c, __dsub_rn(__dmul_rn(d, h), __dmul_rn(e, g)));
    return __dadd_rn(__dsub_rn(t1, t2), t3);
}

// msd from the correlation sums S (row-major 3x3) and the traces.
__device__ __forceinline__ double qcp_msd(const float (&S)[9], double ga, double gb, int n_atoms) {
    const double xx = S[0], xy = S[1], xz = S[2], yx = S[3], yy = S[4], yz = S[5], zx = S[6], zy = S[7], zz = S[8];
    double ss = 0.0;
#pragma unroll
    for (int e = 0; e < 9; ++e) ss = __dadd_rn(ss, __dmul_rn((double)S[e], (double)S[e]));
    const double C2 = __dmul_rn(-2.0, ss);
    const double C1 = __dmul_rn(-8.0, det3_d(xx, xy, xz, yx, yy, yz, zx, zy, zz));
    const double k00 = __dadd_rn(__dadd_rn(xx, yy), zz), k01 = __dsub_rn(yz, zy), k02 = __dsub_rn(zx, xz),
                 k03 = __dsub_rn(xy, yx);
    const double k11 = __dsub_rn(__dsub_rn(xx, yy), zz), k12 = __dadd_rn(xy, yx), k13 = __dadd_rn(zx, xz);
    const double k22 = __dsub_rn(__dadd_rn(-xx, yy), zz), k23 = __dadd_rn(yz, zy);
    const double k33 = __dadd_rn(__dsub_rn(-xx, yy), zz);
    // K is symmetric: K[r][c] = K[c][r].
    const double m0 = det3_d(k11, k12, k13, k12, k22, k23, k13, k23, k33);
    const double m1 = det3_d(k01, k12, k13, k02, k22, k23, k03, k23, k33);
    const double m2 = det3_d(k01, k11, k13, k02, k12, k23, k03, k13, k33);
    const double m3 = det3_d(k01, k11, k12, k02, k12, k22, k03, k13, k23);
    const double C0 = __dsub_rn(__dadd_rn(__dsub_rn(__dmul_rn(k00, m0), __dmul_rn(k01, m1)), __dmul_rn(k02, m2)),
                                __dmul_rn(k03, m3));
    double lam = __dmul_rn(0.5, __dadd_rn(ga, gb));
    const double ub = __dmul_rn((double)__fsqrt_rn(__double2float_rn(__dmul_rn(-1.5, C2))), 1.0 + 1e-6);
    if (ub < lam) lam = ub;
    for (int it = 0; it < 50; ++it) {
        const double l2 = __dmul_rn(lam, lam);
        const double a2 = __dadd_rn(l2, C2);
        const double P = __dadd_rn(__dadd_rn(__dmul_rn(a2, l2), __dmul_rn(C1, lam)), C0);
        const double D = __dadd_rn(__dmul_rn(__dmul_rn(2.0, lam), __dadd_rn(l2, a2)), C1);
        const float Df = __double2float_rn(D);
        if (Df == 0.0f) break;
        // outside float's range (coordinates of order 1e5 and more): the double quotient
        const double step = isinf(Df) ? __ddiv_rn(P, D) : __dmul_rn(P, (double)__frcp_rn(Df));
        const double next = __dsub_rn(lam, step);
        lam = next;
        if (fabs(step) < __dmul_rn(1e-11, fabs(next))) break;
    }
    const double msd = __ddiv_rn(__dsub_rn(__dadd_rn(ga, gb), __dmul_rn(2.0, lam)), (double)n_atoms);
    return msd > 0.0 ? msd : 0.0;
}

// msd of two centered rows, one thread walking both in atom order.
__device__ __forceinline__ double rmsd_msd_rows(const float *__restrict__ a, const float *__restrict__ b, double ga,
                                                double gb, int n_atoms) {
    float S[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) S[e] = 0.0f;
    for (int i = 0; i < n_atoms; ++i) {
        const float a0 = a[3 * i], a1 = a[3 * i + 1], a2 = a[3 * i + 2];
        const float b0 = b[3 * i], b1 = b[3 * i + 1], b2 = b[3 * i + 2];
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
    return qcp_msd(S, ga, gb, n_atoms);
}

}  // namespace km

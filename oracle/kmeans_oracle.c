/*
 * kmeans_oracle.c -- CPU restatement of PyEMMA's k-means discretization path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the CUDA
 * kernels in pyemma_gb300/csrc.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py may load it.  The product path never calls it.
 *
 * What it restates
 * ----------------
 * PyEMMA delegates the arithmetic of this path to the third-party package
 * deeptime (unpinned: setup.py:307 requires deeptime>=0.4.2,
 * devtools/conda-recipe/meta.yaml:38 deeptime>=0.3.0).  deeptime is not part
 * of the reference tree, so this file restates the published behaviour of its
 * call sites:
 *
 *   assign    pyemma/coordinates/clustering/interface.py:157-167
 *             (ClusterModel(centers, metric).transform(X), float32 input,
 *              int32 output).  Squared Euclidean distance, accumulated in
 *              float32 sequentially over features f = 0..d-1, each term
 *              rounded as (x-c), (x-c)*(x-c), acc+term with no fused
 *              multiply-add (the x86-64 baseline build of the reference has
 *              no FMA instructions).  Lowest index wins ties.  A frame whose
 *              every distance is NaN gets label 0.
 *   update    pyemma/coordinates/clustering/kmeans.py:253-258 (KMeans.fit):
 *             new center = mean of members, summed in float64; an empty
 *             cluster keeps its previous center (assumption: deeptime's
 *             behaviour could not be checked, its source is absent).
 *   inertia   kmeans.py:71-75 docstring: C(S) = sum_i sum_{x in S_i}
 *             ||x - mu_i||^2, evaluated in float64 for the new centers and
 *             the assignment of the same iteration.
 *   stopping  kmeans.py:432-436 (the in-repo copy of the rule):
 *             rel = |cost - prev| / cost (0 if cost == 0), prev starts at 0,
 *             converged when rel <= tolerance; at most max_iter iterations.
 *   kmeans++  kmeans.py:211-212,253 (init_strategy='kmeans++', seeded by
 *             fixed_seed, an integer in [0, 2^32-1], kmeans.py:146-164):
 *             first center uniform at random, every later center drawn with
 *             probability proportional to D^2, the squared distance to the
 *             nearest center chosen so far (Arthur & Vassilvitskii 2007).
 *             Random numbers come from Philox4x32-10 (Salmon et al., SC'11);
 *             D^2 weights are quantised to integers so that every prefix sum
 *             is exact and any summation order draws the same center.
 *
 * Parity status: the float order inside deeptime is unpinned (deeptime is
 * absent).  The oracle is pinned by the known-answer tests of the reference
 * (pyemma/coordinates/clustering/tests/test_assign.py and test_kmeans.py),
 * restated in tests/test_oracle_pins.py.
 *
 * Build: gcc -O3 -fopenmp -ffp-contract=off -fPIC -shared (oracle/build.sh).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define KMO_OK 0
#define KMO_BAD_ARG -1
#define KMO_NOMEM -2

int kmo_version(void) { return 1; }

/* ------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: */
/* as easy as 1, 2, 3", SC'11).                                        */
/* ------------------------------------------------------------------ */
void kmo_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* The 64-bit draw of kmeans++ round r: counter (r, 0, tag, 0), key (seed, tag2). */
uint64_t kmo_kmpp_draw(uint32_t seed, uint32_t round) {
    uint32_t ctr[4] = {round, 0u, 0x6B6D7070u, 0u};
    uint32_t key[2] = {seed, 0x4B4D4750u};
    uint32_t out[4];
    kmo_philox4x32_10(ctr, key, out);
    return ((uint64_t)out[0] << 32) | (uint64_t)out[1];
}

static inline uint64_t mulhi64(uint64_t a, uint64_t b) {
    return (uint64_t)(((unsigned __int128)a * (unsigned __int128)b) >> 64);
}

/* Exponent E with 2^(E-1) <= m < 2^E for a positive finite float m. */
static int float_ceil_exp(float m) {
    uint32_t b;
    memcpy(&b, &m, 4);
    int be = (int)((b >> 23) & 0xFFu);
    if (be) return be - 126;
    uint32_t mant = b & 0x7FFFFFu;
    int p = 31 - __builtin_clz(mant);
    return p - 148;
}

/* Scale exponent for the integer D^2 weights: with M the largest finite
 * weight and L = ceil(log2 n), every weight floor(w * 2^e) is below
 * 2^(62-L), so the sum of all n weights stays below 2^62. */
int kmo_quant_exponent(float max_weight, int64_t n) {
    if (!(max_weight > 0.0f) || isinf(max_weight)) return INT32_MIN;
    int L = 0;
    while (((int64_t)1 << L) < n) ++L;
    return 62 - L - float_ceil_exp(max_weight);
}

static inline uint64_t quant_weight(float w, double scale) {
    if (!(w > 0.0f) || isinf(w)) return 0;
    return (uint64_t)((double)w * scale);
}

/* ------------------------------------------------------------------ */
/* Distances                                                          */
/* ------------------------------------------------------------------ */
float kmo_sqdist(const float *x, const float *c, int32_t d) {
    float acc = 0.0f;
    for (int32_t f = 0; f < d; ++f) {
        float t = x[f] - c[f];
        float s = t * t;
        acc = acc + s;
    }
    return acc;
}

/* Centers regrouped in blocks, feature-major inside a block, so that the
 * compiler can evaluate a block's independent sequential sums at once: blocks
 * of 32 centers first, then blocks of 8 for the remainder, then single
 * centers.  Each sum keeps its own feature order, so every distance equals
 * kmo_sqdist's, and the scan visits centers in index order (lowest index on
 * ties). */
#define KMO_CB_WIDE 32
#define KMO_CB_NARROW 8

static float *transpose_center_blocks(const float *C, int32_t k, int32_t d) {
    int32_t nw = k / KMO_CB_WIDE;
    int32_t nn = (k - nw * KMO_CB_WIDE) / KMO_CB_NARROW;
    int32_t kb = nw * KMO_CB_WIDE + nn * KMO_CB_NARROW;
    if (kb == 0) return NULL;
    float *ct = (float *)malloc((size_t)kb * d * sizeof(float));
    if (!ct) return NULL;
    for (int32_t j0 = 0; j0 < kb;) {
        int32_t cb = j0 < nw * KMO_CB_WIDE ? KMO_CB_WIDE : KMO_CB_NARROW;
        float *blk = ct + (size_t)j0 * d;
        for (int32_t f = 0; f < d; ++f)
            for (int32_t u = 0; u < cb; ++u) blk[(size_t)f * cb + u] = C[(size_t)(j0 + u) * d + f];
        j0 += cb;
    }
    return ct;
}

static inline __attribute__((always_inline)) void scan_block(const float *x, int32_t d, const float *blk,
                                                             const int cb, int32_t j0, float *best,
                                                             int32_t *bj) {
    float acc[KMO_CB_WIDE];
    for (int u = 0; u < cb; ++u) acc[u] = 0.0f;
    for (int32_t f = 0; f < d; ++f) {
        float xf = x[f];
        for (int u = 0; u < cb; ++u) {
            float t = xf - blk[(size_t)f * cb + u];
            float s = t * t;
            acc[u] = acc[u] + s;
        }
    }
    for (int u = 0; u < cb; ++u)
        if (acc[u] < *best) {
            *best = acc[u];
            *bj = j0 + u;
        }
}

static void assign_one(const float *x, int32_t d, const float *C, const float *ct, int32_t k,
                       int32_t *label, float *dist) {
    float best = INFINITY;
    int32_t bj = 0;
    int32_t j = 0;
    if (ct) {
        for (; j + KMO_CB_WIDE <= k; j += KMO_CB_WIDE)
            scan_block(x, d, ct + (size_t)j * d, KMO_CB_WIDE, j, &best, &bj);
        for (; j + KMO_CB_NARROW <= k; j += KMO_CB_NARROW)
            scan_block(x, d, ct + (size_t)j * d, KMO_CB_NARROW, j, &best, &bj);
    }
    for (; j < k; ++j) {
        float dd = kmo_sqdist(x, C + (size_t)j * d, d);
        if (dd < best) {
            best = dd;
            bj = j;
        }
    }
    *label = bj;
    if (dist) *dist = best;
}

/* labels[i] = argmin_j D(x_i, c_j); dist (nullable) receives the minimum. */
int kmo_assign(const float *X, int64_t n, int32_t d, const float *C, int32_t k, int32_t *labels,
               float *dist, int32_t n_threads) {
    if (n < 0 || d <= 0 || k <= 0 || (n > 0 && (!X || !labels)) || !C) return KMO_BAD_ARG;
    float *ct = transpose_center_blocks(C, k, d);
    if (n_threads <= 0) n_threads = 1;
#pragma omp parallel for num_threads(n_threads) schedule(static)
    for (int64_t i = 0; i < n; ++i)
        assign_one(X + (size_t)i * d, d, C, ct, k, labels + i, dist ? dist + i : NULL);
    free(ct);
    return KMO_OK;
}

/* ------------------------------------------------------------------ */
/* Centroid update and inertia (float64)                              */
/* ------------------------------------------------------------------ */
/* Sums are taken relative to each cluster's previous center:
 *   S_j = sum_{i in j} (x_i - c_j),  Q_j = sum_{i in j} ||x_i - c_j||^2
 * new center  mu_j = float(c_j + S_j / n_j)     (c_j kept when n_j == 0)
 * inertia_j   = Q_j - 2 delta_j . S_j + n_j ||delta_j||^2,  delta_j = mu_j - c_j
 * which is sum_{i in j} ||x_i - mu_j||^2 evaluated in float64.  Frames are
 * visited in index order. */
int kmo_update(const float *X, int64_t n, int32_t d, const int32_t *labels, int32_t k,
               const float *C_old, float *C_new, int64_t *counts, double *cost_out,
               double *cluster_cost) {
    if (n < 0 || d <= 0 || k <= 0 || !C_old || !C_new || !counts) return KMO_BAD_ARG;
    double *S = (double *)calloc((size_t)k * d, sizeof(double));
    double *Q = (double *)calloc((size_t)k, sizeof(double));
    if (!S || !Q) {
        free(S);
        free(Q);
        return KMO_NOMEM;
    }
    memset(counts, 0, (size_t)k * sizeof(int64_t));
    for (int64_t i = 0; i < n; ++i) {
        int32_t j = labels[i];
        if (j < 0 || j >= k) {
            free(S);
            free(Q);
            return KMO_BAD_ARG;
        }
        const float *x = X + (size_t)i * d;
        const float *c = C_old + (size_t)j * d;
        double *s = S + (size_t)j * d;
        double q = 0.0;
        for (int32_t f = 0; f < d; ++f) {
            double t = (double)x[f] - (double)c[f];
            s[f] += t;
            q += t * t;
        }
        Q[j] += q;
        counts[j] += 1;
    }
    double cost = 0.0;
    for (int32_t j = 0; j < k; ++j) {
        const float *c = C_old + (size_t)j * d;
        float *m = C_new + (size_t)j * d;
        double cj = 0.0;
        if (counts[j] == 0) {
            memmove(m, c, (size_t)d * sizeof(float));
        } else {
            double cnt = (double)counts[j];
            const double *s = S + (size_t)j * d;
            double cross = 0.0, sq = 0.0;
            for (int32_t f = 0; f < d; ++f) {
                float mu = (float)((double)c[f] + s[f] / cnt);
                double dl = (double)mu - (double)c[f];
                cross += dl * s[f];
                sq += dl * dl;
                m[f] = mu;
            }
            cj = Q[j] - 2.0 * cross + cnt * sq;
        }
        if (cluster_cost) cluster_cost[j] = cj;
        cost += cj;
    }
    *cost_out = cost;
    free(S);
    free(Q);
    return KMO_OK;
}

/* ------------------------------------------------------------------ */
/* Lloyd iterations                                                   */
/* ------------------------------------------------------------------ */
int kmo_lloyd(const float *X, int64_t n, int32_t d, int32_t k, float *C, int32_t max_iter,
              double tol, int32_t *labels, double *inertias, int32_t *n_iter, int32_t *converged,
              int32_t n_threads) {
    if (n <= 0 || d <= 0 || k <= 0 || !C || !labels || max_iter < 0) return KMO_BAD_ARG;
    float *Cn = (float *)malloc((size_t)k * d * sizeof(float));
    int64_t *cnt = (int64_t *)malloc((size_t)k * sizeof(int64_t));
    if (!Cn || !cnt) {
        free(Cn);
        free(cnt);
        return KMO_NOMEM;
    }
    double prev = 0.0;
    int32_t it = 0, conv = 0;
    int rc = KMO_OK;
    while (it < max_iter) {
        rc = kmo_assign(X, n, d, C, k, labels, NULL, n_threads);
        if (rc) break;
        double cost;
        rc = kmo_update(X, n, d, labels, k, C, Cn, cnt, &cost, NULL);
        if (rc) break;
        memcpy(C, Cn, (size_t)k * d * sizeof(float));
        if (inertias) inertias[it] = cost;
        double rel = cost != 0.0 ? fabs(cost - prev) / cost : 0.0;
        prev = cost;
        ++it;
        if (rel <= tol) {
            conv = 1;
            break;
        }
    }
    free(Cn);
    free(cnt);
    if (n_iter) *n_iter = it;
    if (converged) *converged = conv;
    return rc;
}

/* ------------------------------------------------------------------ */
/* kmeans++                                                           */
/* ------------------------------------------------------------------ */
int kmo_kmpp(const float *X, int64_t n, int32_t d, int32_t k, uint32_t seed, float *C0,
             int64_t *idx_out, int32_t n_threads) {
    if (n <= 0 || d <= 0 || k <= 0 || !X || !C0) return KMO_BAD_ARG;
    if (n_threads <= 0) n_threads = 1;
    int64_t p = (int64_t)mulhi64(kmo_kmpp_draw(seed, 0), (uint64_t)n);
    memcpy(C0, X + (size_t)p * d, (size_t)d * sizeof(float));
    if (idx_out) idx_out[0] = p;
    if (k == 1) return KMO_OK;
    float *mind = (float *)malloc((size_t)n * sizeof(float));
    if (!mind) return KMO_NOMEM;
#pragma omp parallel for num_threads(n_threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) mind[i] = kmo_sqdist(X + (size_t)i * d, C0, d);
    float M = 0.0f;
    for (int64_t i = 0; i < n; ++i)
        if (isfinite(mind[i]) && mind[i] > M) M = mind[i];
    int e = kmo_quant_exponent(M, n);
    double scale = (e == INT32_MIN) ? 0.0 : ldexp(1.0, e);
    for (int32_t r = 1; r < k; ++r) {
        if (r >= 2) {
            const float *c = C0 + (size_t)(r - 1) * d;
#pragma omp parallel for num_threads(n_threads) schedule(static)
            for (int64_t i = 0; i < n; ++i) {
                float dd = kmo_sqdist(X + (size_t)i * d, c, d);
                if (dd < mind[i]) mind[i] = dd;
            }
        }
        uint64_t total = 0;
#pragma omp parallel for num_threads(n_threads) schedule(static) reduction(+ : total)
        for (int64_t i = 0; i < n; ++i) total += quant_weight(mind[i], scale);
        uint64_t r64 = kmo_kmpp_draw(seed, (uint32_t)r);
        if (total == 0) {
            p = (int64_t)mulhi64(r64, (uint64_t)n);
        } else {
            uint64_t t = mulhi64(r64, total);
            uint64_t acc = 0;
            p = n - 1;
            for (int64_t i = 0; i < n; ++i) {
                acc += quant_weight(mind[i], scale);
                if (acc > t) {
                    p = i;
                    break;
                }
            }
        }
        memcpy(C0 + (size_t)r * d, X + (size_t)p * d, (size_t)d * sizeof(float));
        if (idx_out) idx_out[r] = p;
    }
    free(mind);
    return KMO_OK;
}

/* Regular space clustering, first pass (pyemma/coordinates/clustering/
 * regspace.py:140-152, deeptime RegularSpace.partial_fit over the chunks in
 * iteration order): the first frame becomes a center; every later frame
 * becomes one when its distance to every center so far is at least dmin.
 * Distance: sqrtf of the float32 sequential squared distance (kmo_sqdist),
 * compared in double with dmin (assumption: deeptime's exact comparison
 * could not be checked; pyemma's comment reads ">= dmin").  Stops when a
 * (max_centers+1)-th center would be added.  Returns the number of centers
 * in *n_centers and 1 in *converged unless max_centers was hit. */
int kmo_regspace(const float *X, int64_t n, int32_t d, double dmin, int32_t max_centers, float *centers,
                 int32_t *n_centers, int32_t *converged) {
    int32_t nc = 0;
    *converged = 1;
    for (int64_t i = 0; i < n; ++i) {
        const float *x = X + i * d;
        int is_new = 1;
        for (int32_t j = 0; j < nc; ++j) {
            const float dist = sqrtf(kmo_sqdist(x, centers + (int64_t)j * d, d));
            if (!((double)dist >= dmin)) {
                is_new = 0;
                break;
            }
        }
        if (is_new) {
            if (nc == max_centers) {
                *converged = 0;
                break;
            }
            memcpy(centers + (int64_t)nc * d, x, sizeof(float) * (size_t)d);
            ++nc;
        }
    }
    *n_centers = nc;
    return 0;
}

/* ------------------------------------------------------------------ */
/* minRMSD metric                                                     */
/* ------------------------------------------------------------------ */
/* The minRMSD metric of pyemma/coordinates/clustering/src/
 * clustering_module.cpp:9-36 (RMSDMetric, registered into deeptime's
 * clustering): frames are atom-major (x0 y0 z0 x1 ...), d = 3 n_atoms; the
 * squared metric is the mean square deviation after optimal translation and
 * rotation, found with the quaternion characteristic polynomial method
 * (Theobald, Acta Cryst. A61:478-480, 2005; mdtraj's libtheobald, which the
 * reference links).  mdtraj is absent, so its float order is unpinned; this
 * restatement fixes one order, which the CUDA kernels follow operation for
 * operation:
 *
 *   centering  per row, the per-axis sum over atoms in double in the order of
 *              a 32-lane warp: lane l sums atoms l, l+32, ... in turn, then an
 *              xor butterfly (offsets 16, 8, 4, 2, 1) adds the lanes; the mean
 *              is that sum / n_atoms; a = (float)(x - mean).  G = sum of a^2
 *              (double products, double sums) in the same lane order.
 *   pair       S[p][q] = sum_i a_i[p] b_i[q], float fused multiply-adds in atom
 *              order; then in double: C2 = -2 sum S^2, C1 = -8 det S,
 *              C0 = det K (the 4x4 key matrix, Laplace expansion on row 0);
 *              Newton on P = lambda^4 + C2 lambda^2 + C1 lambda + C0 from
 *              the smaller of two upper bounds of the largest root,
 *              (Ga + Gb) / 2 and sqrt(3) ||S||_F = sqrt(-1.5 C2) (a float
 *              root inflated by 1e-6), at most 50 steps, until
 *              |step| < 1e-11 |lambda|,
 *              with P and P' in double and the step P * r, r the float
 *              reciprocal of (float)P', or P / P' when that is outside float's
 *              range (the root is P's; the derivative only
 *              scales the step, and a double division costs too much on the
 *              GPU's FP64 pipe);
 *              msd = max(0, (Ga + Gb - 2 lambda) / n_atoms).
 *   assign     the lowest-index minimum of msd (NaN never wins; label 0 when
 *              no msd is a number).
 *   update     the mean of the members (kmo_update: deeptime's center update
 *              does not depend on the metric); inertia = sum_i msd(x_i,
 *              new center of its label) (assumption: deeptime's cost for a
 *              custom metric could not be checked).
 *   kmeans++   D^2 sampling with D^2 = (float)msd, the draws of kmo_kmpp. */

static double butterfly32(double s[32]) {
    double t[32];
    for (int off = 16; off > 0; off >>= 1) {
        for (int l = 0; l < 32; ++l) t[l] = s[l] + s[l ^ off];
        memcpy(s, t, sizeof(t));
    }
    return s[0];
}

/* Centers one atom-major row (n_atoms = d / 3) into a; returns G. */
double kmo_rmsd_center(const float *x, int32_t n_atoms, float *a) {
    double mean[3];
    for (int c = 0; c < 3; ++c) {
        double s[32];
        for (int l = 0; l < 32; ++l) {
            double acc = 0.0;
            for (int32_t i = l; i < n_atoms; i += 32) acc += (double)x[3 * i + c];
            s[l] = acc;
        }
        mean[c] = butterfly32(s) / (double)n_atoms;
    }
    double g[32];
    for (int l = 0; l < 32; ++l) {
        double acc = 0.0;
        for (int32_t i = l; i < n_atoms; i += 32)
            for (int c = 0; c < 3; ++c) {
                const float v = (float)((double)x[3 * i + c] - mean[c]);
                acc += (double)v * (double)v;
            }
        g[l] = acc;
    }
    for (int32_t i = 0; i < n_atoms; ++i)
        for (int c = 0; c < 3; ++c) a[3 * i + c] = (float)((double)x[3 * i + c] - mean[c]);
    return butterfly32(g);
}

static double det3(double a, double b, double c, double d, double e, double f, double g, double h, double i) {
    return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}

/* msd of two centered rows a, b with traces ga, gb. */
double kmo_rmsd_msd(const float *a, const float *b, double ga, double gb, int32_t n_atoms) {
    float S[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int32_t i = 0; i < n_atoms; ++i)
        for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q) S[3 * p + q] = fmaf(a[3 * i + p], b[3 * i + q], S[3 * p + q]);
    const double xx = S[0], xy = S[1], xz = S[2], yx = S[3], yy = S[4], yz = S[5], zx = S[6], zy = S[7], zz = S[8];
    double ss = 0.0;
    for (int e = 0; e < 9; ++e) ss += (double)S[e] * (double)S[e];
    const double C2 = -2.0 * ss;
    const double C1 = -8.0 * det3(xx, xy, xz, yx, yy, yz, zx, zy, zz);
    const double K[4][4] = {{xx + yy + zz, yz - zy, zx - xz, xy - yx},
                            {yz - zy, xx - yy - zz, xy + yx, zx + xz},
                            {zx - xz, xy + yx, -xx + yy - zz, yz + zy},
                            {xy - yx, zx + xz, yz + zy, -xx - yy + zz}};
    const double m0 = det3(K[1][1], K[1][2], K[1][3], K[2][1], K[2][2], K[2][3], K[3][1], K[3][2], K[3][3]);
    const double m1 = det3(K[1][0], K[1][2], K[1][3], K[2][0], K[2][2], K[2][3], K[3][0], K[3][2], K[3][3]);
    const double m2 = det3(K[1][0], K[1][1], K[1][3], K[2][0], K[2][1], K[2][3], K[3][0], K[3][1], K[3][3]);
    const double m3 = det3(K[1][0], K[1][1], K[1][2], K[2][0], K[2][1], K[2][2], K[3][0], K[3][1], K[3][2]);
    const double C0 = K[0][0] * m0 - K[0][1] * m1 + K[0][2] * m2 - K[0][3] * m3;
    double lam = 0.5 * (ga + gb);
    const double ub = (double)sqrtf((float)(-1.5 * C2)) * (1.0 + 1e-6);
    if (ub < lam) lam = ub;
    for (int it = 0; it < 50; ++it) {
        const double l2 = lam * lam;
        const double a2 = l2 + C2;
        const double P = (a2 * l2 + C1 * lam) + C0;
        const double D = (2.0 * lam) * (l2 + a2) + C1;
        const float Df = (float)D;
        if (Df == 0.0f) break;
        /* outside float's range (coordinates of order 1e5 and more): the double quotient */
        const double step = isinf(Df) ? P / D : P * (double)(1.0f / Df);
        const double next = lam - step;
        lam = next;
        if (fabs(step) < 1e-11 * fabs(next)) break;
    }
    const double msd = ((ga + gb) - 2.0 * lam) / (double)n_atoms;
    return msd > 0.0 ? msd : 0.0;
}

/* Centers every row of an (n, d) array (d = 3 n_atoms). */
static int rmsd_center_all(const float *X, int64_t n, int32_t d, float **Xc, double **G, int32_t n_threads) {
    *Xc = (float *)malloc((size_t)n * d * sizeof(float));
    *G = (double *)malloc((size_t)n * sizeof(double));
    if (!*Xc || !*G) {
        free(*Xc);
        free(*G);
        return KMO_NOMEM;
    }
#pragma omp parallel for num_threads(n_threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) (*G)[i] = kmo_rmsd_center(X + (size_t)i * d, d / 3, *Xc + (size_t)i * d);
    return KMO_OK;
}

int kmo_assign_minrmsd(const float *X, int64_t n, int32_t d, const float *C, int32_t k, int32_t *labels,
                       double *msd_out, int32_t n_threads) {
    if (n < 0 || d <= 0 || d % 3 || k <= 0 || !C || !labels) return KMO_BAD_ARG;
    if (n == 0) return KMO_OK;
    if (n_threads <= 0) n_threads = 1;
    float *Xc, *Cc;
    double *G, *H;
    int rc = rmsd_center_all(X, n, d, &Xc, &G, n_threads);
    if (rc) return rc;
    rc = rmsd_center_all(C, k, d, &Cc, &H, n_threads);
    if (rc) {
        free(Xc);
        free(G);
        return rc;
    }
#pragma omp parallel for num_threads(n_threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double best = 0.0;
        int32_t bj = -1;
        for (int32_t j = 0; j < k; ++j) {
            const double m = kmo_rmsd_msd(Xc + (size_t)i * d, Cc + (size_t)j * d, G[i], H[j], d / 3);
            if (m == m && (bj < 0 || m < best)) {
                best = m;
                bj = j;
            }
        }
        labels[i] = bj < 0 ? 0 : bj;
        if (msd_out) msd_out[i] = bj < 0 ? NAN : best;
    }
    free(Xc);
    free(G);
    free(Cc);
    free(H);
    return KMO_OK;
}

/* rmsd = sqrt(msd) of row pairs (X[i], Y[i]), as compute_metric returns it. */
int kmo_minrmsd_rows(const float *X, const float *Y, int64_t n, int32_t d, float *out) {
    if (n < 0 || d <= 0 || d % 3) return KMO_BAD_ARG;
    float *a = (float *)malloc((size_t)d * sizeof(float));
    float *b = (float *)malloc((size_t)d * sizeof(float));
    if (!a || !b) {
        free(a);
        free(b);
        return KMO_NOMEM;
    }
    for (int64_t i = 0; i < n; ++i) {
        const double ga = kmo_rmsd_center(X + (size_t)i * d, d / 3, a);
        const double gb = kmo_rmsd_center(Y + (size_t)i * d, d / 3, b);
        out[i] = (float)sqrt(kmo_rmsd_msd(a, b, ga, gb, d / 3));
    }
    free(a);
    free(b);
    return KMO_OK;
}

/* inertia of an assignment under the metric: sum_i msd(x_i, C[labels[i]]). */
static double minrmsd_cost(const float *X, int64_t n, int32_t d, const float *C, int32_t k, const int32_t *labels,
                           int32_t n_threads) {
    float *Cc;
    double *H;
    if (rmsd_center_all(C, k, d, &Cc, &H, n_threads)) return NAN;
    double cost = 0.0;
    float *a = (float *)malloc((size_t)d * sizeof(float));
    for (int64_t i = 0; i < n; ++i) {
        const double g = kmo_rmsd_center(X + (size_t)i * d, d / 3, a);
        const int32_t j = labels[i];
        cost += kmo_rmsd_msd(a, Cc + (size_t)j * d, g, H[j], d / 3);
    }
    free(a);
    free(Cc);
    free(H);
    return cost;
}

/* Regular space clustering under the minRMSD metric (regspace.py:89
 * registers the metric, regspace.py:144-152 walks the frames;
 * test_regspace.py:107-115,137-141 run it): kmo_regspace's walk with the
 * distance rmsd = (float)sqrt(msd(frame, center)) (the frame's centered row
 * first in the correlation sums, as in kmo_assign_minrmsd), compared in
 * double with dmin.  Centers are the frames' own (uncentered) rows. */
int kmo_regspace_minrmsd(const float *X, int64_t n, int32_t d, double dmin, int32_t max_centers, float *centers,
                         int32_t *n_centers, int32_t *converged) {
    if (n < 0 || d <= 0 || d % 3 || max_centers < 1 || !n_centers || !converged) return KMO_BAD_ARG;
    *n_centers = 0;
    *converged = 1;
    if (n == 0) return KMO_OK;
    float *Xc;
    double *G;
    int rc = rmsd_center_all(X, n, d, &Xc, &G, 1);
    if (rc) return rc;
    int64_t *idx = (int64_t *)malloc((size_t)max_centers * sizeof(int64_t));
    if (!idx) {
        free(Xc);
        free(G);
        return KMO_NOMEM;
    }
    int32_t nc = 0;
    for (int64_t i = 0; i < n; ++i) {
        int is_new = 1;
        for (int32_t j = 0; j < nc; ++j) {
            const int64_t c = idx[j];
            const float dist = (float)sqrt(kmo_rmsd_msd(Xc + (size_t)i * d, Xc + (size_t)c * d, G[i], G[c], d / 3));
            if (!((double)dist >= dmin)) {
                is_new = 0;
                break;
            }
        }
        if (is_new) {
            if (nc == max_centers) {
                *converged = 0;
                break;
            }
            idx[nc] = i;
            memcpy(centers + (size_t)nc * d, X + (size_t)i * d, sizeof(float) * (size_t)d);
            ++nc;
        }
    }
    *n_centers = nc;
    free(idx);
    free(Xc);
    free(G);
    return KMO_OK;
}

int kmo_lloyd_minrmsd(const float *X, int64_t n, int32_t d, int32_t k, float *C, int32_t max_iter, double tol,
                      int32_t *labels, double *inertias, int32_t *n_iter, int32_t *converged, int32_t n_threads) {
    if (n <= 0 || d <= 0 || d % 3 || k <= 0 || !C || !labels || max_iter < 0) return KMO_BAD_ARG;
    float *Cn = (float *)malloc((size_t)k * d * sizeof(float));
    int64_t *cnt = (int64_t *)malloc((size_t)k * sizeof(int64_t));
    if (!Cn || !cnt) {
        free(Cn);
        free(cnt);
        return KMO_NOMEM;
    }
    double prev = 0.0;
    int32_t it = 0, conv = 0;
    int rc = KMO_OK;
    while (it < max_iter) {
        rc = kmo_assign_minrmsd(X, n, d, C, k, labels, NULL, n_threads);
        if (rc) break;
        double unused;
        rc = kmo_update(X, n, d, labels, k, C, Cn, cnt, &unused, NULL);
        if (rc) break;
        memcpy(C, Cn, (size_t)k * d * sizeof(float));
        const double cost = minrmsd_cost(X, n, d, C, k, labels, n_threads);
        if (inertias) inertias[it] = cost;
        double rel = cost != 0.0 ? fabs(cost - prev) / cost : 0.0;
        prev = cost;
        ++it;
        if (rel <= tol) {
            conv = 1;
            break;
        }
    }
    free(Cn);
    free(cnt);
    if (n_iter) *n_iter = it;
    if (converged) *converged = conv;
    return rc;
}

int kmo_kmpp_minrmsd(const float *X, int64_t n, int32_t d, int32_t k, uint32_t seed, float *C0, int64_t *idx_out,
                     int32_t n_threads) {
    if (n <= 0 || d <= 0 || d % 3 || k <= 0 || !X || !C0) return KMO_BAD_ARG;
    if (n_threads <= 0) n_threads = 1;
    float *Xc;
    double *G;
    int rc = rmsd_center_all(X, n, d, &Xc, &G, n_threads);
    if (rc) return rc;
    int64_t p = (int64_t)mulhi64(kmo_kmpp_draw(seed, 0), (uint64_t)n);
    memcpy(C0, X + (size_t)p * d, (size_t)d * sizeof(float));
    if (idx_out) idx_out[0] = p;
    float *mind = (float *)malloc((size_t)n * sizeof(float));
    if (!mind) {
        free(Xc);
        free(G);
        return KMO_NOMEM;
    }
    int64_t last = p;
    double scale = 0.0;
    for (int32_t r = 1; r < k; ++r) {
#pragma omp parallel for num_threads(n_threads) schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            const float dd = (float)kmo_rmsd_msd(Xc + (size_t)i * d, Xc + (size_t)last * d, G[i], G[last], d / 3);
            if (r == 1 || dd < mind[i]) mind[i] = dd;
        }
        if (r == 1) {
            float M = 0.0f;
            for (int64_t i = 0; i < n; ++i)
                if (isfinite(mind[i]) && mind[i] > M) M = mind[i];
            int e = kmo_quant_exponent(M, n);
            scale = (e == INT32_MIN) ? 0.0 : ldexp(1.0, e);
        }
        uint64_t total = 0;
        for (int64_t i = 0; i < n; ++i) total += quant_weight(mind[i], scale);
        uint64_t r64 = kmo_kmpp_draw(seed, (uint32_t)r);
        if (total == 0) {
            p = (int64_t)mulhi64(r64, (uint64_t)n);
        } else {
            uint64_t t = mulhi64(r64, total);
            uint64_t acc = 0;
            p = n - 1;
            for (int64_t i = 0; i < n; ++i) {
                acc += quant_weight(mind[i], scale);
                if (acc > t) {
                    p = i;
                    break;
                }
            }
        }
        memcpy(C0 + (size_t)r * d, X + (size_t)p * d, (size_t)d * sizeof(float));
        if (idx_out) idx_out[r] = p;
        last = p;
    }
    free(mind);
    free(Xc);
    free(G);
    return KMO_OK;
}

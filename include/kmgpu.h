/*
 * kmgpu.h -- C ABI of the GB300 k-means discretization library (libkmgpu.so).
 *
 * The library replaces the native layer under PyEMMA's clustering estimators.
 * In the reference that layer is deeptime's pybind11 module, reached from
 *   pyemma/coordinates/clustering/kmeans.py:211-214, 253-258
 *       KMeans(n_clusters, max_iter, metric, tolerance, init_strategy,
 *              fixed_seed, n_jobs).fit(X, callback_init_centers,
 *              callback_loop).fetch_model()
 *   pyemma/coordinates/clustering/interface.py:157-167
 *       ClusterModel(cluster_centers, metric).transform(X)
 * Each entry point below names the reference call it stands in for.
 *
 * Conventions
 *   - Every array pointer is a DEVICE pointer owned by the caller, except
 *     where a parameter says "host".  Frames are row-major float32 (n, d);
 *     centers are row-major float32 (k, d); labels are int32.
 *   - Scratch memory is a caller-owned device workspace whose size the
 *     matching *_workspace_size() function returns; pass NULL/0 when it
 *     returns 0.  Entry points allocate no device memory of their own,
 *     except the two object constructors: km_centers_create (a resident
 *     center set) and km_serve_create (the serving loop's batch slots).
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  Work is
 *     enqueued on it; calls that return host results synchronise it.
 *   - Every call returns a km_status; km_last_error() gives a message for
 *     the last failing call on the calling thread.
 *   - 1 <= d <= 4096, 1 <= k <= 1048576, 0 <= n < 2^31.
 */
#ifndef KMGPU_H
#define KMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    KM_OK = 0,
    KM_ERR_BAD_SHAPE = 1,       /* a size is out of range or a required pointer is NULL */
    KM_ERR_WORKSPACE = 2,       /* workspace missing or smaller than *_workspace_size() */
    KM_ERR_NON_FINITE = 3,      /* the input holds NaN or infinity where that is not allowed */
    KM_ERR_TIMEOUT = 4,         /* a bounded device-side wait expired; the context stays usable */
    KM_ERR_CUDA = 5,            /* a CUDA runtime call failed */
    KM_ERR_UNSUPPORTED = 6,     /* the requested precision or shape has no kernel on this device */
    KM_ERR_BAD_LABEL = 7,       /* a label is outside [0, k) */
    KM_PENDING = 8              /* km_serve_poll: the request has not completed yet (not an error) */
} km_status;

/* Distance arithmetic of the assignment.
 *   KM_PREC_FP32: exact float32 difference of squares in feature order
 *                 (plain CUDA-core kernel).
 *   KM_PREC_FP16: tensor-core distances (tcgen05, FP16 operands scaled by a
 *                 power of two, FP32 accumulate) with an exact FP32 recheck
 *                 of every frame whose nearest centers lie within the derived
 *                 error bound; the labels equal the KM_PREC_FP32 labels bit
 *                 for bit.
 *   KM_PREC_BF16: the same with BF16 operands (8-bit mantissa: a wider bound,
 *                 so more frames are re-checked; same labels).
 *   KM_PREC_FP8:  the same with FP8 e4m3 operands (tcgen05 kind::f8f6f4):
 *                 each frame scaled by its own power of two, the centers by
 *                 one; the center norms are applied in the epilogue.  A
 *                 3-bit mantissa makes the bound wide, so most frames are
 *                 re-checked; same labels.
 *   KM_PREC_AUTO: the library picks by (d, k) (km_tune can measure it). */
typedef enum {
    KM_PREC_FP32 = 0,
    KM_PREC_FP16 = 1,
    KM_PREC_AUTO = 2,
    KM_PREC_BF16 = 3,
    KM_PREC_FP8 = 4
} km_precision;

/* Progress hook, called on the calling host thread (kmeans.py:241-251
 * passes callback_init_centers / callback_loop into the native fit). */
typedef void (*km_callback)(void *user);

/* Counters of one assignment (host struct, filled when a pointer is given). */
typedef struct {
    int64_t n_frames;   /* frames assigned */
    int64_t n_recheck;  /* frames re-evaluated exactly over their candidate list */
    int64_t n_full;     /* frames re-evaluated exactly over all k centers */
    int64_t n_flipped;  /* frames whose exact label differs from the tensor-core argmin */
    int32_t precision;  /* precision actually used (km_precision) */
    int32_t reserved;
    int64_t n_pairs;    /* (frame, candidate center) pairs listed for the exact re-check */
} km_assign_stats;

int km_version(void);
const char *km_status_string(int status);
const char *km_last_error(void);

/* ---- kernel timing with CUDA events (diagnostics; no reference counterpart)
 * km_profile_enable(1) resets the totals and makes later km_assign /
 * km_lloyd calls record an event pair around their main kernels, including
 * inside CUDA-graph replays; the pair is read at the synchronisation points
 * these calls already have.  kind: 0 tensor-core distance kernel, 1 exact
 * FP32 assignment kernel, 2 exact recheck of candidate pairs, 3 centroid
 * update, 4 exact recheck of frames over all centers.
 * km_profile_read returns the summed milliseconds and the launch count. */
int km_profile_enable(int on);
int km_profile_read(int32_t kind, double *ms_total, int64_t *launches);

/* ---- test hook (diagnostics; no reference counterpart) --------------------
 * The next km_update or km_update_noalloc call ORs `bits` into the device
 * error word it reads back, as if a kernel had set them (1, 2, 4: a
 * device-side wait ran out; 8: a label out of range), and returns the
 * status that word maps to.  Lets tests check the mapping without making a
 * device wait run out. */
int km_debug_fake_device_error(uint32_t bits);

/* ---- assignment: ClusterModel(centers, 'euclidean').transform(X) ----------
 * interface.py:157-167.  labels[i] = argmin_j ||X[i]-C[j]||^2, float32
 * distances summed in feature order, lowest index on ties.  stats (host,
 * nullable) synchronises the stream.  The tensor-core forms read labels
 * before they write it: a value in [0, k) seeds the frame's search (a
 * previous labelling makes it faster where k >= 2048 and d <= 126); the
 * result does not depend on what the array held, and the array need not be
 * initialised. */
size_t km_assign_workspace_size(int64_t n, int32_t d, int32_t k, int32_t precision);
int km_assign(const float *X, int64_t n, int32_t d, const float *C, int32_t k, int32_t precision,
              int32_t *labels, void *workspace, size_t workspace_bytes, km_assign_stats *stats,
              void *stream);

/* ---- diagnostics: tensor-core distances (no reference counterpart) --------
 * Runs the assignment in a tensor-core precision (KM_PREC_FP16, KM_PREC_BF16
 * or KM_PREC_FP8; labels as km_assign).  V (device, n*k
 * floats, nullable) receives the tensor-core approximation of every squared
 * distance, V[i*k + j]; the tests use it to check the error bound pair by
 * pair.  wait_cycles (host, 8 counters, nullable) receives the SM cycles the
 * kernel's roles spent waiting: producer on free B / A buffers, MMA issuer on
 * loaded B / A and on a drained accumulator, epilogue on a ready
 * accumulator, then the epilogue's and the MMA issuer's total cycles.
 * Workspace as km_assign with KM_PREC_FP16 (enough for every tensor-core
 * precision). */
int km_debug_tc_distances(const float *X, int64_t n, int32_t d, const float *C, int32_t k, int32_t precision,
                          float *V, int32_t *labels, uint64_t *wait_cycles, void *workspace, size_t workspace_bytes,
                          void *stream);

/* ---- batched assignment of uneven trajectories --------------------------
 * The get_output loop of datasource.py:402-406 runs transform chunk by chunk
 * and trajectory by trajectory.  Here all trajectories, packed back to back
 * in X_packed, go through one launch.  offsets (host, n_traj+1 entries,
 * offsets[0] = 0, non-decreasing) delimit trajectory t as frames
 * [offsets[t], offsets[t+1]).  Workspace as km_assign with n = offsets[n_traj]. */
int km_batch_assign(const float *X_packed, const int64_t *offsets, int32_t n_traj, int32_t d,
                    const float *C, int32_t k, int32_t precision, int32_t *labels_packed,
                    void *workspace, size_t workspace_bytes, km_assign_stats *stats, void *stream);

/* ---- one centroid update: the M-step inside KMeans.fit -------------------
 * kmeans.py:253-258.  C_new[j] = mean of frames labelled j (float64 sums);
 * an empty cluster keeps C_old[j].  cost (device, 1 double) receives the
 * inertia sum_i ||X[i] - C_new[labels[i]]||^2 in float64; counts (device,
 * k int64, nullable) the cluster sizes.  C_new must not alias C_old. */
size_t km_update_workspace_size(int64_t n, int32_t d, int32_t k);
int km_update(const float *X, int64_t n, int32_t d, const int32_t *labels, int32_t k,
              const float *C_old, float *C_new, int64_t *counts, double *cost, void *workspace,
              size_t workspace_bytes, void *stream);

/* ---- centroid update without a workspace (no counterpart in the reference) --
 * Same arithmetic, outputs and statuses as km_update, for callers that
 * cannot provide device memory (a plugin inside a host program that owns all
 * device allocations, or a loop that must not call cudaMalloc).  Its scratch
 * is a fixed array inside the library of km_update_noalloc_max_bytes() bytes
 * (32 MiB), held on every GPU that loads the library until the process
 * exits.  A shape fits when km_update_workspace_size(n, d, k) is at most that
 * (8 n + 8 k d + 32 k bytes plus about 2.5 KB of alignment, so n up to about
 * 4 million frames at small k d); larger shapes return KM_ERR_WORKSPACE.  The
 * first call on a device looks up the array's device address.  Every call
 * reads the device error word back and synchronises `stream`, so it must not
 * be called on a stream that is being captured: it returns
 * KM_ERR_UNSUPPORTED there, before enqueuing anything.  Calls on one device
 * share that device's array, so the library runs them one at a time: a call
 * holds that device's lock from its first launch until `stream` has drained.
 * Calls on different devices do not wait for each other. */
size_t km_update_noalloc_max_bytes(void);
int km_update_noalloc(const float *X, int64_t n, int32_t d, const int32_t *labels, int32_t k,
                      const float *C_old, float *C_new, int64_t *counts, double *cost, void *stream);

/* ---- kmeans++ initialisation: KMeans(init_strategy='kmeans++') -----------
 * kmeans.py:211-212,253; seed = fixed_seed (kmeans.py:146-164).  Writes k
 * centers into C0 (device, k*d floats) and, when idx is given (device, k
 * int64), the chosen frame indices.  cb (nullable) fires once per center. */
size_t km_kmpp_workspace_size(int64_t n, int32_t d, int32_t k);
int km_kmpp(const float *X, int64_t n, int32_t d, int32_t k, uint32_t seed, float *C0, int64_t *idx,
            km_callback cb, void *cb_user, void *workspace, size_t workspace_bytes, void *stream);

/* ---- Lloyd iterations: KMeans.fit from given centers ---------------------
 * kmeans.py:253-258 (fit), stopping rule as kmeans.py:432-436.  C (device,
 * k*d) holds the initial centers and receives the final ones.  labels
 * (device, n) receives the assignment of the last iteration.  inertias
 * (host, max_iter doubles, nullable), n_iter and converged (host) report the
 * run.  Each iteration is one CUDA-graph launch; cb fires after each. */
size_t km_lloyd_workspace_size(int64_t n, int32_t d, int32_t k, int32_t precision);
int km_lloyd(const float *X, int64_t n, int32_t d, int32_t k, float *C, int32_t max_iter,
             double tolerance, int32_t precision, int32_t *labels, double *inertias,
             int32_t *n_iter, int32_t *converged, km_callback cb, void *cb_user, void *workspace,
             size_t workspace_bytes, void *stream);

/* km_lloyd on frames that are still in host memory: X_parts[q] (host,
 * part_rows[q] x d row-major float32) are copied one after the other into X
 * (device, n x d, caller-owned; it holds the frames afterwards), in chunks on
 * a stream of the library's own.  The first iteration assigns each chunk as
 * soon as its copy has landed, so the transfer and the assignment overlap;
 * the run is otherwise km_lloyd's (same workspace, results equal to km_lloyd
 * on the copied X).  Where the GPU reads host memory in place
 * (cudaDevAttrPageableMemoryAccess) a device kernel copies every part,
 * page-locked or pageable, on a stream of the device's greatest priority
 * (its CTAs claim 16 KB blocks in turn, so a CTA placed late behind the
 * assignment's CTAs does not hold back a chunk); elsewhere page-locked parts go through the copy
 * engines and pageable ones through worker threads and page-locked blocks;
 * all forms overlap.  With max_iter = 0 it only copies.  Stands in for the same fit as km_lloyd, reached with
 * frames that the reference holds in host memory (kmeans.py:253-258 with the
 * in-memory chunks that kmeans.py:218-234 and 326-338 gather). */
int km_lloyd_host(const float *const *X_parts, const int64_t *part_rows, int32_t n_parts, float *X, int64_t n,
                  int32_t d, int32_t k, float *C, int32_t max_iter, double tolerance, int32_t precision,
                  int32_t *labels, double *inertias, int32_t *n_iter, int32_t *converged, km_callback cb,
                  void *cb_user, void *workspace, size_t workspace_bytes, void *stream);

/* ---- the minRMSD metric ----------------------------------------------------
 * Stands in for the minRMSD metric plug-in of
 * pyemma/coordinates/clustering/src/clustering_module.cpp:9-36 (RMSDMetric,
 * registered into deeptime's clustering; reached by cluster_kmeans(...,
 * metric='minRMSD') and assign_to_centers(..., metric='minRMSD')).  Rows are
 * atom-major (x0 y0 z0 x1 ...), d = 3 n_atoms; other d give
 * KM_ERR_BAD_SHAPE, as the reference raises.  The squared metric is the mean
 * square deviation after optimal translation and rotation (Theobald's
 * quaternion characteristic polynomial).
 *
 * km_assign_minrmsd: labels (device, n) of the lowest-index center with the
 *   smallest msd; rmsd (device, n, nullable) receives sqrt(msd) as float.
 * km_minrmsd_rows: rmsd[i] = the metric of the row pair (X[i], Y[i])
 *   (compute_metric, clustering_module.cpp:41-43).
 * km_kmpp_minrmsd: kmeans++ with D^2 = msd (km_kmpp's draws); C0 receives
 *   the chosen frames (uncentered), idx (device, nullable) their indexes.
 * km_lloyd_minrmsd: Lloyd iterations as km_lloyd, assigning by the metric;
 *   the new center is the mean of its members, the inertia the sum of the
 *   members' msd to the new centers. */
size_t km_assign_minrmsd_workspace_size(int64_t n, int32_t d, int32_t k);
int km_assign_minrmsd(const float *X, int64_t n, int32_t d, const float *C, int32_t k, int32_t *labels, float *rmsd,
                      void *workspace, size_t workspace_bytes, void *stream);
size_t km_minrmsd_rows_workspace_size(int64_t n, int32_t d);
int km_minrmsd_rows(const float *X, const float *Y, int64_t n, int32_t d, float *rmsd, void *workspace,
                    size_t workspace_bytes, void *stream);
size_t km_kmpp_minrmsd_workspace_size(int64_t n, int32_t d, int32_t k);
int km_kmpp_minrmsd(const float *X, int64_t n, int32_t d, int32_t k, uint32_t seed, float *C0, int64_t *idx,
                    km_callback cb, void *cb_user, void *workspace, size_t workspace_bytes, void *stream);
size_t km_lloyd_minrmsd_workspace_size(int64_t n, int32_t d, int32_t k);
int km_lloyd_minrmsd(const float *X, int64_t n, int32_t d, int32_t k, float *C, int32_t max_iter, double tolerance,
                     int32_t *labels, double *inertias, int32_t *n_iter, int32_t *converged, km_callback cb,
                     void *cb_user, void *workspace, size_t workspace_bytes, void *stream);

/* ---- precision autotuning (no counterpart in the reference) ---------------
 * KM_PREC_AUTO picks the faster of the exact FP32 kernel and the tensor-core
 * path by a rule measured on a d x k sweep.  km_tune measures instead: it
 * times both on the given frames and centers (one warm-up and three timed
 * km_assign calls each; the caller passes a representative sample) and
 * stores the faster for this (d, k) in a process-wide table behind a mutex,
 * which KM_PREC_AUTO consults first.  chosen, ms_fp32 and ms_fp16 (host,
 * nullable) receive the choice and the per-call times (ms_fp16 = -1 when the
 * tensor-core path has no kernel for the shape).  Synchronises `stream`;
 * refuses to run while the stream is being captured.  km_tune_clear empties
 * the table. */
size_t km_tune_workspace_size(int64_t n, int32_t d, int32_t k);
int km_tune(const float *X, int64_t n, int32_t d, const float *C, int32_t k, void *workspace,
            size_t workspace_bytes, int32_t *chosen, double *ms_fp32, double *ms_fp16, void *stream);
int km_tune_clear(void);

/* ---- tile-shape autotuning (no counterpart in the reference) --------------
 * The tensor-core kernel's tile shape: bn center columns per tile (64, 128
 * or 256; k rounded up to 32 below that), pair = 1 for the CTA-pair form
 * (tcgen05 cta_group::2, M = 256 frames over two SMs; bn = 256 only),
 * stages of its TMA ring, and list_len candidates kept per frame (8 or 16;
 * a frame with more near-ties goes to the exact re-check over all centers).
 * Every shape gives the same labels.  km_tune_tiles times every shape that
 * fits (d, k) on the given frames and centers (one warm-up and three timed
 * km_assign calls each, precision KM_PREC_FP16 or KM_PREC_BF16), writes
 * the fastest to *best and up to max_tried timed shapes to tried (host,
 * nullable; *n_tried gets their number), and stores the fastest in a
 * process-wide table behind a mutex: later tensor-core calls for (d, k)
 * use it (km_tune_clear empties the table).  Workspace as km_tune.
 * Synchronises `stream`; refuses to run while the stream is captured.
 * km_tile_plan_get reports the shape that FP16 calls for (d, k) use now
 * (*tuned = 1 when it comes from the table).  Without a stored shape, FP16
 * keeps 8 candidates per frame up to d = 256 and 16 above; BF16 and FP8
 * keep 16. */
typedef struct {
    int32_t bn, pair, stages, list_len;
    double ms; /* mean time of one km_assign call with this shape (km_tune_tiles) */
} km_tile_plan;
int km_tune_tiles(const float *X, int64_t n, int32_t d, const float *C, int32_t k, int32_t precision,
                  void *workspace, size_t workspace_bytes, km_tile_plan *best, km_tile_plan *tried,
                  int32_t max_tried, int32_t *n_tried, void *stream);
int km_tile_plan_get(int32_t d, int32_t k, km_tile_plan *plan, int32_t *tuned);

/* Test hook (diagnostics): tensor-core calls of the calling host thread use
 * `plan` until the hook is called with NULL; a shape that does not fit
 * makes them return KM_ERR_UNSUPPORTED. */
int km_debug_force_tile_plan(const km_tile_plan *plan);

/* ---- regular space clustering, first pass ----------------------------------
 * RegularSpaceClustering._estimate, pyemma/coordinates/clustering/
 * regspace.py:140-152 (deeptime RegularSpace.partial_fit).  Walks the n
 * frames of X in order: the first becomes a center, a later one becomes a
 * center when its distance (sqrt of the float32 squared distance in feature
 * order, correctly rounded) to every center so far is >= dmin.  centers
 * (device, max_centers*d floats) receives them, *n_centers (host) their
 * number.  When a (max_centers+1)-th center would be added the walk stops
 * and *converged (host) is 0 (the reference's MaxCentersReached case).
 * Synchronises `stream` once per 65,536 frames. */
size_t km_regspace_workspace_size(int32_t d);
int km_regspace(const float *X, int64_t n, int32_t d, double dmin, int32_t max_centers, float *centers,
                int32_t *n_centers, int32_t *converged, void *workspace, size_t workspace_bytes, void *stream);

/* ---- lag-tau transition counts of discrete trajectories ---------------------
 * The step after discretization: pyemma/msm/estimators/_dtraj_stats.py:139-145
 * (deeptime count_matrix / TransitionCountEstimator).  dtrajs (device int32)
 * holds the trajectories back to back, delimited by offsets (host, n_traj+1
 * entries, offsets[0] = 0).  counts (device, nstates*nstates int64,
 * row-major from -> to) receives, per trajectory, the pairs
 * (dtraj[t], dtraj[t+lag]) for t = 0 .. T-lag-1 (sliding != 0) or
 * t = 0, lag, 2 lag, ... < T-lag (sliding == 0); pairs with a state outside
 * [0, nstates) (e.g. -1, unassigned) are left out. */
size_t km_count_matrix_workspace_size(int32_t n_traj);
int km_count_matrix(const int32_t *dtrajs, const int64_t *offsets, int32_t n_traj, int32_t lag, int32_t sliding,
                    int32_t nstates, int64_t *counts, void *workspace, size_t workspace_bytes, void *stream);

/* ---- atom-pair distance features --------------------------------------------
 * The featurization that feeds the discretization:
 * pyemma/coordinates/data/featurization/featurizer.py:305-372 (add_distances,
 * add_distances_ca) and distances.py:53-54 (mdtraj.compute_distances, no
 * unit cell).  xyz (device, n * n_atoms * 3 float32, frame-major), pairs
 * (device, npairs * 2 int32 atom indices), out (device, n * npairs float32):
 * out[t*npairs + p] = sqrt((dx*dx + dy*dy) + dz*dz) in float32 with
 * d = xyz[t, pairs[p][1]] - xyz[t, pairs[p][0]].  The pair table is read
 * back and checked on the host first (KM_ERR_BAD_SHAPE for an atom index
 * outside [0, n_atoms)), which synchronises `stream`. */
int km_pair_distances(const float *xyz, int64_t n, int32_t n_atoms, const int32_t *pairs, int32_t npairs,
                      float *out, void *stream);

/* ---- frames given as atom coordinates: the featurization fused in ---------
 * The reference featurizes on the host (featurizer.py:305-372 add_distances
 * / add_distances_ca -> distances.py:53-54 mdtraj.compute_distances) and
 * hands (T, n_pairs) float32 features to the clustering; km_pair_distances
 * does that step on the device.  These calls skip it: they take the
 * coordinates xyz (device, n x n_atoms x 3 float32, frame-major) and the
 * atom pairs (device, d x 2 int32, every index in [0, n_atoms), checked on
 * the host after a read-back of the d x 2 table), and every kernel that
 * needs a float32 feature computes it where it reads it, with the
 * arithmetic of km_pair_distances, so no n x d feature matrix is ever
 * written.  Results equal km_assign / km_lloyd / km_kmpp on the output of
 * km_pair_distances, bit for bit (labels, kmeans++ draws) or to the
 * rounding of the float64 centroid sums (centers, inertia).  Workspaces are
 * those of the dense calls with the same n, d, k.  KM_PREC_FP8 is not built
 * for coordinate frames (KM_ERR_UNSUPPORTED). */
size_t km_assign_pairs_workspace_size(int64_t n, int32_t d, int32_t k, int32_t precision);
int km_assign_pairs(const float *xyz, int64_t n, int32_t n_atoms, const int32_t *pairs, int32_t d, const float *C,
                    int32_t k, int32_t precision, int32_t *labels, void *workspace, size_t workspace_bytes,
                    km_assign_stats *stats, void *stream);
size_t km_lloyd_pairs_workspace_size(int64_t n, int32_t d, int32_t k, int32_t precision);
int km_lloyd_pairs(const float *xyz, int64_t n, int32_t n_atoms, const int32_t *pairs, int32_t d, int32_t k,
                   float *C, int32_t max_iter, double tolerance, int32_t precision, int32_t *labels,
                   double *inertias, int32_t *n_iter, int32_t *converged, km_callback cb, void *cb_user,
                   void *workspace, size_t workspace_bytes, void *stream);
size_t km_kmpp_pairs_workspace_size(int64_t n, int32_t d, int32_t k);
int km_kmpp_pairs(const float *xyz, int64_t n, int32_t n_atoms, const int32_t *pairs, int32_t d, int32_t k,
                  uint32_t seed, float *C0, int64_t *idx, km_callback cb, void *cb_user, void *workspace,
                  size_t workspace_bytes, void *stream);

/* ---- resident center sets: ClusterModel(centers, metric) built once -------
 * interface.py:164-165 constructs ClusterModel(cluster_centers, metric) for
 * every chunk it transforms.  A km_centers handle holds a device copy of
 * the centers and, for KM_PREC_FP16, their scaled FP16 copy, norms and
 * centering shift, prepared once; any number of km_assign_centers calls on
 * any streams may share it.  km_centers_create copies C (device), resolves
 * KM_PREC_AUTO, allocates the device memory that km_centers_info reports
 * and synchronises `stream`.  km_centers_destroy frees it; no call using
 * the handle may still be running. */
typedef struct km_centers km_centers;
int km_centers_create(const float *C, int32_t k, int32_t d, int32_t precision, void *stream, km_centers **out);
int km_centers_destroy(km_centers *centers);
int km_centers_info(const km_centers *centers, int32_t *k, int32_t *d, int32_t *precision,
                    int64_t *device_bytes);

/* Assignment against a resident set: labels as km_assign with the set's
 * precision.  The workspace holds only the per-frame buffers. */
size_t km_assign_centers_workspace_size(int64_t n, const km_centers *centers);
int km_assign_centers(const float *X, int64_t n, int32_t d, const km_centers *centers, int32_t *labels,
                      void *workspace, size_t workspace_bytes, km_assign_stats *stats, void *stream);

/* ---- serving loop (no counterpart in the reference) ------------------------
 * A native worker thread assigns trajectories submitted from any host
 * thread against resident center sets.  Requests for the same center set
 * are packed into one batch (continuous batching); the batch is led by the
 * queued request with the fewest frames left, or by the oldest request once
 * it has waited 25 ms, and filled with the other requests of the leader's
 * set, fewest frames left first.  A request longer than a batch is split
 * across batches.  A batch holds at most 64 MiB of frames (or
 * max_batch_frames frames), so short requests do not queue behind the copy
 * of a long one.  Three batch slots rotate so that the copies of one batch
 * overlap the kernels of the others.  The slots (frames, labels, assignment
 * workspace) are the device memory held for requests in flight; their total
 * stays within hbm_budget_bytes.
 *   km_serve_submit: X_host (host, n*d float32) and labels_host (host, n
 *     int32) must stay valid until the request completes.  Where the GPU
 *     reads host memory in place a device kernel copies the frames, from
 *     any host memory; elsewhere page-locked buffers let the copies run
 *     asynchronously.  d must match the set.
 *   km_serve_poll: waits up to timeout_ms (-1: no limit) for the request;
 *     returns KM_PENDING if it has not completed, else its final status,
 *     after which the ticket is released.  info (host, nullable) receives
 *     its timings.
 *   km_serve_shutdown: completes every submitted request, stops the worker
 *     and frees the slots.  The center sets stay owned by the caller. */
typedef struct {
    int64_t hbm_budget_bytes;  /* device bytes for requests in flight; 0 = 40 GiB */
    int64_t max_batch_frames;  /* frames per batch at most; 0 = as many as the budget allows */
    int32_t device;            /* CUDA device of the server */
    int32_t reserved;
} km_serve_config;

typedef struct {
    int32_t status;       /* km_status of the request (KM_PENDING while running) */
    int32_t set_id;
    int64_t n_frames;
    int64_t batch_frames; /* frames of the largest batch the request ran in */
    double queue_ms;      /* submit -> launch of its first batch */
    double total_ms;      /* submit -> its labels in host memory */
} km_request_info;

typedef struct {
    int64_t batches;          /* batches launched */
    int64_t frames;           /* frames assigned */
    int64_t requests;         /* requests completed */
    int64_t batch_cap_frames; /* frames per batch allowed by the budget */
    int64_t device_bytes;     /* device memory held by the batch slots */
} km_serve_stats;

typedef struct km_server km_server;
int km_serve_create(const km_serve_config *config, km_server **out);
int km_serve_add_centers(km_server *server, const km_centers *centers, int32_t *set_id);
int km_serve_submit(km_server *server, int32_t set_id, const float *X_host, int64_t n, int32_t d,
                    int32_t *labels_host, uint64_t *ticket);
int km_serve_poll(km_server *server, uint64_t ticket, int32_t timeout_ms, km_request_info *info);
int km_serve_stats_read(km_server *server, km_serve_stats *stats);
int km_serve_shutdown(km_server *server);

#ifdef __cplusplus
}
#endif

#endif /* KMGPU_H */

"""Pins the CPU oracle to the known answers of the reference's own tests.

The reference's k-means arithmetic (deeptime) is absent, so the oracle is a
restatement; these tests re-express the reference's known-answer tests with
freshly generated inputs and run them against it.  Each test names the
reference test it follows.
"""
import numpy as np
import pytest


def _kmeans(O, X, k, seed=42, max_iter=10, tol=1e-5, C0=None):
    X = np.asarray(X, dtype=np.float32)
    if X.ndim == 1:
        X = X[:, None]
    if C0 is None:
        C0, _ = O.kmpp(X, k, seed)
    return O.lloyd(X, np.asarray(C0, dtype=np.float32), max_iter, tol)


def test_philox_known_answers(oracle, golden):
    for c, k, o in zip(golden["philox_ctr"], golden["philox_key"], golden["philox_out"]):
        assert oracle.philox4x32_10(list(c), list(k)) == list(o)


def test_assign_five_blobs_exact(oracle):
    # test_assign.py:50-78,102-109: dtraj[i] == i // 1000 for separated blobs.
    rng = np.random.default_rng(1)
    means = np.array([[-3, 0], [-1, 1], [0, 0], [1, -1], [4, 2]], dtype=float)
    X = np.zeros((5000, 2))
    for i in range(5):
        X[i * 1000:(i + 1) * 1000] = 0.1 * rng.normal(size=(1000, 2)) + means[i]
    labels = oracle.assign(X, means.astype(np.float32))
    assert labels.dtype == np.int32
    np.testing.assert_array_equal(labels, np.arange(5000) // 1000)


def test_assign_thread_invariance(oracle):
    # test_assign.py:232-239: multithreaded == single-threaded assignment.
    rng = np.random.default_rng(2)
    X = rng.normal(size=(5000, 2)).astype(np.float32)
    C = X[rng.choice(5000, 100)]
    np.testing.assert_array_equal(oracle.assign(X, C, n_threads=1), oracle.assign(X, C, n_threads=4))


def test_kmeans_k1_cube_is_origin(oracle):
    # test_kmeans.py:154-166: k=1 on the 8 cube corners gives exactly (0,0,0).
    X = np.array([[1, 1, 1], [1, 1, -1], [1, -1, -1], [-1, -1, -1], [-1, 1, 1], [-1, -1, 1], [-1, 1, -1],
                  [1, -1, 1]], dtype=np.float32)
    r = _kmeans(oracle, X, 1)
    np.testing.assert_equal(r["centers"].squeeze(), np.zeros(3))


def test_kmeans_outlier_converges(oracle):
    # test_kmeans.py:168-179: from (+-2,0,0), max_iter=500, all |centers| <= 1.
    X = np.array([[1, 1.5, 1], [1, 1, -1], [1, -1, -1], [-1, -1, -1], [-1, 1, 1], [-1, -1, 1], [-1, 1, -1],
                  [1, -1, 1]], dtype=np.float32)
    r = _kmeans(oracle, X, 2, C0=[[2, 0, 0], [-2, 0, 0]], max_iter=500)
    assert np.all(np.abs(r["centers"]) <= 1)


def test_kmeans_convex_hull(oracle):
    # test_kmeans.py:181-233: the k=1 center is the mean, inside the hull.
    rng = np.random.default_rng(3)
    P = rng.normal(size=(24, 3)).astype(np.float32)
    r = _kmeans(oracle, P, 1)
    np.testing.assert_allclose(r["centers"][0], P.astype(np.float64).mean(0), rtol=0, atol=1e-6)


def test_kmeans_trivial_blocks_exact(oracle):
    # test_kmeans.py:411-426: four constant blocks -> centers exactly 30/60/90/120.
    X = np.zeros((40000, 4), dtype=np.float32)
    for b, v in enumerate((30.0, 60.0, 90.0, 120.0)):
        X[b * 10000:(b + 1) * 10000] = v
    r = _kmeans(oracle, X, 4, seed=42)
    found = sorted(float(c[0]) for c in r["centers"] if np.all(c == c[0]))
    assert found == [30.0, 60.0, 90.0, 120.0]


def test_kmeans_seeded_determinism(oracle):
    # test_kmeans.py:64-102: same seed -> identical initial and final centers.
    rng = np.random.default_rng(42)
    X = np.hstack([rng.normal(size=200) - 2.0, rng.normal(size=200), rng.normal(size=200) + 2.0])[:, None]
    X = X.astype(np.float32)
    for seed in (42, 463498):
        a, ia = oracle.kmpp(X, 50, seed)
        b, ib = oracle.kmpp(X, 50, seed)
        np.testing.assert_equal(a, b)
        ra = _kmeans(oracle, X, 50, C0=a, max_iter=100)
        rb = _kmeans(oracle, X, 50, C0=b, max_iter=100)
        np.testing.assert_allclose(ra["centers"], rb["centers"], atol=1e-6)
        cc = ra["centers"]
        assert np.all(np.isfinite(cc)) and np.any((cc > -1.0) & (cc < 1.0))


def test_kmeans_serial_equals_parallel(oracle):
    # test_kmeans.py:104-128: n_jobs=1 and n_jobs=2 give the same centers.
    rng = np.random.default_rng(45)
    means = rng.uniform(-10, 10, size=(6, 2))
    X = np.concatenate([m + 0.5 * rng.normal(size=(84, 2)) for m in means]).astype(np.float32)
    C0, _ = oracle.kmpp(X, 6, 7)
    a = oracle.lloyd(X, C0, 50, 1e-5, n_threads=1)
    b = oracle.lloyd(X, C0, 50, 1e-5, n_threads=2)
    np.testing.assert_allclose(a["centers"], b["centers"], atol=1e-4)


def test_kmeans_resume_reduces_error(oracle):
    # test_kmeans.py:357-374: resuming from 1-iteration centers moves them towards (-2, 0, 2).
    rng = np.random.default_rng(32)
    X = np.hstack([rng.normal(size=1000) - 2.0, rng.normal(size=1000), rng.normal(size=1000) + 2.0])
    X = X[:, None].astype(np.float32)
    r1 = oracle.lloyd(X, np.array([[20], [42], [-29]], dtype=np.float32), 1, 1e-5)
    r2 = oracle.lloyd(X, r1["centers"], 50, 1e-5)
    true = np.array([-2, 0, 2])
    d0 = np.linalg.norm(true - np.sort(r1["centers"].ravel()))
    d1 = np.linalg.norm(true - np.sort(r2["centers"].ravel()))
    assert d1 < d0


def test_stopping_rule_first_iteration(oracle):
    # kmeans.py:432-436: prev starts at 0, so the first iteration never converges
    # unless the inertia is 0.
    X = np.array([[0.0], [0.0], [5.0], [5.0]], dtype=np.float32)
    r = oracle.lloyd(X, np.array([[0.0], [5.0]], dtype=np.float32), 10, 1e-5)
    assert r["n_iter"] == 1 and r["converged"] and r["inertias"][0] == 0.0
    X2 = np.array([[0.0], [1.0], [5.0], [6.0]], dtype=np.float32)
    r2 = oracle.lloyd(X2, np.array([[0.0], [5.0]], dtype=np.float32), 10, 1e-5)
    assert r2["n_iter"] == 2 and r2["converged"]
    np.testing.assert_allclose(r2["inertias"], [1.0, 1.0])


def test_empty_cluster_keeps_center(oracle):
    X = np.array([[0.0, 0.0], [0.1, 0.0]], dtype=np.float32)
    C = np.array([[0.0, 0.0], [100.0, 100.0]], dtype=np.float32)
    labels = oracle.assign(X, C)
    Cn, counts, cost, _ = oracle.update(X, labels, C)
    assert counts.tolist() == [2, 0]
    np.testing.assert_array_equal(Cn[1], C[1])


def test_update_matches_float64_reference(oracle):
    rng = np.random.default_rng(5)
    X = (1000.0 + rng.normal(size=(4000, 9))).astype(np.float32)
    C = X[:30].copy()
    lab = oracle.assign(X, C)
    Cn, counts, cost, _ = oracle.update(X, lab, C)
    C64, cnt = oracle.centers_fp64(X, lab, C)
    np.testing.assert_allclose(Cn, C64, rtol=1e-7, atol=0)
    np.testing.assert_array_equal(counts, cnt.astype(np.int64))
    assert abs(cost - oracle.inertia_fp64(X, lab, Cn)) <= 1e-9 * cost


def test_kmpp_spreads_centers(oracle):
    # D^2 sampling on 4 far-apart tight blobs picks one center per blob.
    rng = np.random.default_rng(9)
    means = np.array([[0, 0], [100, 0], [0, 100], [100, 100]], dtype=float)
    X = np.concatenate([m + 0.01 * rng.normal(size=(500, 2)) for m in means]).astype(np.float32)
    for seed in range(5):
        C, idx = oracle.kmpp(X, 4, seed)
        assert sorted(set(int(i) // 500 for i in idx)) == [0, 1, 2, 3]


def test_kmpp_duplicate_data_falls_back_to_uniform(oracle):
    X = np.ones((50, 3), dtype=np.float32)
    C, idx = oracle.kmpp(X, 5, 11)
    assert C.shape == (5, 3) and np.all(C == 1.0)
    assert np.all((idx >= 0) & (idx < 50))


def test_quant_exponent_bounds(oracle):
    for M, n in [(1.0, 1), (3.5, 1000), (1e-30, 2 ** 31 - 1), (1e30, 7), (1.4e-45, 100)]:
        e = oracle.quant_exponent(M, n)
        M = float(np.float32(M))
        L = int(np.ceil(np.log2(n))) if n > 1 else 0
        assert M * 2.0 ** e < 2.0 ** (62 - L)
        assert M * 2.0 ** e >= 2.0 ** (61 - L)


@pytest.mark.parametrize("d", [1, 2, 3, 8, 9, 33])
def test_assign_matches_sequential_numpy(oracle, d):
    rng = np.random.default_rng(d)
    X = rng.normal(size=(500, d)).astype(np.float32)
    C = rng.normal(size=(19, d)).astype(np.float32)
    D = oracle.sqdist_fp32_sequential(X, C)
    lab, dist = oracle.assign(X, C, return_dist=True)
    np.testing.assert_array_equal(lab, np.argmin(D, axis=1))
    np.testing.assert_array_equal(dist, D.min(axis=1))


def test_regspace_oracle_properties(oracle):
    # regspace.py docstring and reference test_regspace.py: centers at least
    # dmin apart, the first frame is the first center, max_centers stops the walk.
    import itertools
    rng = np.random.default_rng(11)
    X = rng.random((1000, 3)).astype(np.float32)
    C, conv = oracle.regspace(X, 0.3, 1000)
    assert conv and len(C) > 1
    np.testing.assert_array_equal(C[0], X[0])
    for a, b in itertools.combinations(C, 2):
        assert np.linalg.norm(a - b) >= 0.3
    # every frame is within dmin of some center (else it would be one)
    d = np.sqrt(((X[:, None, :].astype(np.float64) - C[None].astype(np.float64)) ** 2).sum(-1)).min(1)
    assert (d < 0.3 + 1e-6).all()
    C2, conv2 = oracle.regspace(X, 1e-8, 50)
    assert not conv2 and len(C2) == 50
    np.testing.assert_array_equal(C2, X[:50])


def test_count_matrix_oracle_known_answers(oracle):
    # sliding: T - lag pairs (t, t+lag); sample: pairs at multiples of lag
    # (the count modes documented at pyemma/msm/estimators/_dtraj_stats.py:103-117)
    d = np.array([0, 0, 1, 1, 0])
    C = oracle.count_matrix([d], 1)
    np.testing.assert_array_equal(C, [[1, 1], [1, 1]])
    C = oracle.count_matrix([d], 2, sliding=False)
    np.testing.assert_array_equal(C, [[0, 1], [1, 0]])
    C = oracle.count_matrix([np.array([0, -1, 1, 1]), np.array([2])], 1)
    np.testing.assert_array_equal(C, [[0, 0, 0], [0, 1, 0], [0, 0, 0]])


# ---------------------------------------------------------------------------
# minRMSD metric (clustering_module.cpp:9-36); the reference's tests are
# test_kmeans.py:235-316 and test_assign.py:241-274
# ---------------------------------------------------------------------------
def _rotation(axis, theta):
    axis = np.asarray(axis, dtype=np.float64)
    axis = axis / np.linalg.norm(axis)
    a = np.cos(theta / 2.0)
    b, c, d = -axis * np.sin(theta / 2.0)
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c + a * d), 2 * (b * d - a * c)],
                     [2 * (b * c - a * d), a * a + c * c - b * b - d * d, 2 * (c * d + a * b)],
                     [2 * (b * d + a * c), 2 * (c * d - a * b), a * a + d * d - b * b - c * c]])


def rotated_clusters(rng, n_clusters=5, n_particles=3, per_cluster=25):
    """Clusters of one noisy structure each, every frame randomly rotated about
    y and translated (the data of test_kmeans.py:272-299)."""
    out = np.zeros((n_clusters * per_cluster, 3 * n_particles))
    for i in range(n_clusters):
        base = rng.choice(np.arange(3 * n_particles), size=3 * n_particles).astype(float)
        pos = np.repeat(base[None], per_cluster, axis=0) + rng.normal(size=(per_cluster, 3 * n_particles), scale=.1)
        for n, p in enumerate(pos):
            r = _rotation([0, 1, 0], np.pi * rng.random())
            t = rng.normal(size=3)
            for m in range(n_particles):
                out[per_cluster * i + n, 3 * m:3 * (m + 1)] = r @ p[3 * m:3 * (m + 1)] - t
    return out.astype(np.float32)


@pytest.mark.parametrize("n_atoms", [1, 2, 3, 15, 58, 100])
def test_minrmsd_metric_matches_kabsch(oracle, n_atoms):
    # test_kmeans.py:254-265 compares the metric with mdtraj.rmsd (absent
    # here); the float64 Kabsch superposition is the independent check.
    rng = np.random.default_rng(n_atoms)
    X = rng.uniform(size=(20, 3 * n_atoms)).astype(np.float32)
    Y = rng.uniform(size=(20, 3 * n_atoms)).astype(np.float32)
    got = oracle.minrmsd_rows(X, Y)
    ref = np.array([oracle.kabsch_rmsd_fp64(x, y) for x, y in zip(X, Y)])
    np.testing.assert_allclose(got, ref, rtol=2e-5, atol=1e-6)


def test_minrmsd_invariant_under_rigid_motion(oracle):
    rng = np.random.default_rng(4)
    x = rng.normal(size=(40, 3))
    y = x + 0.3 * rng.normal(size=x.shape)
    r = _rotation([0.3, -1.0, 0.5], 1.1)
    y2 = y @ r.T + np.array([4.0, -2.0, 7.0])
    a = oracle.minrmsd_rows(x.astype(np.float32).ravel(), y.astype(np.float32).ravel())[0]
    b = oracle.minrmsd_rows(x.astype(np.float32).ravel(), y2.astype(np.float32).ravel())[0]
    assert abs(a - b) <= 1e-5 * a
    assert abs(a - oracle.kabsch_rmsd_fp64(x, y)) <= 1e-5 * a


def test_minrmsd_assignment_is_argmin_of_metric(oracle):
    # test_kmeans.py:235-252: kmeans++ (seeded) is deterministic and the
    # assignment is the argmin of the metric to the centers.
    rng = np.random.RandomState(123)
    data = rng.uniform(-50, 50, size=(500, 3 * 15)).astype(np.float32)
    C1, i1 = oracle.kmpp_minrmsd(data, 15, 32)
    C2, i2 = oracle.kmpp_minrmsd(data, 15, 32)
    np.testing.assert_array_equal(i1, i2)
    labels = oracle.assign_minrmsd(data, C1)
    manual = [int(np.argmin(oracle.minrmsd_rows(np.repeat(f[None], 15, axis=0), C1))) for f in data]
    np.testing.assert_array_equal(labels, manual)


def test_minrmsd_rotated_clusters_assigned(oracle):
    # test_kmeans.py:267-316: every cluster of rotated copies gets one label.
    rng = np.random.default_rng(7)
    out = rotated_clusters(rng)
    C, idx = oracle.kmpp_minrmsd(out, 5, 11)
    labels = oracle.assign_minrmsd(out, C)
    for i in range(5):
        assert len(np.unique(labels[25 * i:25 * (i + 1)])) == 1


def test_minrmsd_lloyd_inertia_decreases(oracle):
    rng = np.random.default_rng(9)
    out = rotated_clusters(rng, n_clusters=6, n_particles=4, per_cluster=40)
    C0, _ = oracle.kmpp_minrmsd(out, 6, 3)
    r = oracle.lloyd_minrmsd(out, C0, 20, 1e-9)
    assert r["n_iter"] >= 1
    assert np.all(np.diff(r["inertias"]) <= 1e-6 * r["inertias"][0])


def test_regspace_minrmsd_oracle(oracle):
    # test_regspace.py:107-115,137-141 run regular space under minRMSD: the
    # walk equals a frame-by-frame loop over compute_metric, the centers are
    # pairwise at least dmin apart, and single atoms (d = 3) are all at
    # distance 0 after centering, so one center remains.
    rng = np.random.default_rng(21)
    X = rotated_clusters(rng, n_clusters=4, n_particles=4, per_cluster=30)
    X = np.concatenate([X, rng.uniform(-2, 2, size=(60, 12)).astype(np.float32)])
    for dmin, max_centers in ((0.9, 1000), (0.5, 1000), (0.5, 7)):
        C, conv = oracle.regspace_minrmsd(X, dmin, max_centers)
        want, full = [], True
        for i in range(len(X)):
            if all(float(oracle.minrmsd_rows(X[i:i + 1], X[c:c + 1])[0]) >= dmin for c in want):
                if len(want) == max_centers:
                    full = False
                    break
                want.append(i)
        np.testing.assert_array_equal(C, X[want])
        assert conv == full
        for a in range(len(C)):
            for b in range(a):
                assert float(oracle.minrmsd_rows(C[a:a + 1], C[b:b + 1])[0]) >= dmin
    assert not oracle.regspace_minrmsd(X, 0.5, 7)[1]
    one_atom = np.random.default_rng(2).uniform(-2, 2, size=(1000, 3)).astype(np.float32)
    C1, conv1 = oracle.regspace_minrmsd(one_atom, 2.0, 1000)
    assert conv1 and len(C1) == 1


def test_lloyd_matches_scikit_learn(oracle):
    # Independent cross-check of the update step: from the same initial
    # centers on well-separated data (float32 and float64 labels agree),
    # n oracle iterations give scikit-learn's Lloyd centers up to float32
    # rounding, and the fixed point's inertia.
    cluster = pytest.importorskip("sklearn.cluster")
    rng = np.random.default_rng(31)
    means = rng.uniform(-6, 6, size=(8, 5))
    X = (means[rng.integers(0, 8, 4000)] + 0.6 * rng.normal(size=(4000, 5))).astype(np.float32)
    C0 = X[rng.choice(4000, 8, replace=False)].copy()
    for iters in (1, 3, 10, 50):
        ref = oracle.lloyd(X, C0, iters, -1.0)
        km = cluster.KMeans(n_clusters=8, init=C0.astype(np.float64), n_init=1, max_iter=iters, tol=0.0,
                            algorithm="lloyd").fit(X.astype(np.float64))
        np.testing.assert_allclose(ref["centers"], km.cluster_centers_, rtol=0, atol=1e-5)
    assert abs(ref["inertias"][-1] - km.inertia_) <= 1e-6 * km.inertia_

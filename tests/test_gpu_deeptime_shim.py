"""The deeptime.clustering-shaped module on the GPU, against the CPU oracle,
called the way PyEMMA's estimators call deeptime (kmeans.py:211-258,
400-426, interface.py:164-165, regspace.py:144-170, test_kmeans.py:247-316).

Bars as in test_gpu_parity.py: labels, kmeans++ centers and regular space
centers bit-exact; Lloyd runs with the same iteration count, centers within
1e-5 and inertias within 1e-6 relative; one mini-batch step's centers within
1e-6 relative.
"""
import numpy as np
import pytest

from test_oracle_pins import rotated_clusters

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dc():
    from pyemma_gb300 import _lib, deeptime_clustering
    _lib.load()
    return deeptime_clustering


def mixture(n, d, comps, seed):
    from pyemma_gb300 import datasets
    return datasets.gaussian_mixture(n, d, comps, 0.4, 5.0, seed)


def test_kmeans_fit_as_pyemma_calls_it(dc, oracle):
    X = mixture(6000, 4, 12, 1)
    inits, loops = [], []
    est = dc.KMeans(20, 60, "euclidean", tolerance=1e-5, init_strategy="kmeans++", fixed_seed=42, n_jobs=1)
    est.fit(X, callback_init_centers=lambda: inits.append(1), callback_loop=lambda: loops.append(1), n_jobs=1)
    model = est.fetch_model()
    C0, _ = oracle.kmpp(X, 20, 42)
    ref = oracle.lloyd(X, C0, 60, 1e-5)
    assert len(inits) == 20
    assert len(model.inertias) == ref["n_iter"] == len(loops)
    assert model.converged == ref["converged"]
    np.testing.assert_allclose(model.cluster_centers, ref["centers"], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(model.inertias, ref["inertias"], rtol=1e-6)
    assert model.cluster_centers.dtype == np.float32
    labels = model.transform(X)
    assert labels.dtype == np.int32 and labels.shape == (6000,)
    np.testing.assert_array_equal(labels, oracle.assign(X, model.cluster_centers))


def test_kmeans_given_centers_and_uniform(dc, oracle):
    X = mixture(3000, 3, 8, 2)
    C0 = X[::300].copy()  # 10 centers
    est = dc.KMeans(10, 30, tolerance=1e-5)
    est.initial_centers = C0  # kmeans.py:213-214: given centers skip the initialisation
    model = est.fit(X).fetch_model()
    ref = oracle.lloyd(X, C0, 30, 1e-5)
    assert len(model.inertias) == ref["n_iter"]
    np.testing.assert_allclose(model.cluster_centers, ref["centers"], rtol=1e-5, atol=1e-5)
    with pytest.raises(ValueError):
        dc.KMeans(11, initial_centers=C0).fit(X)
    u1 = dc.KMeans(10, 0, init_strategy="uniform", fixed_seed=5).fit(X).fetch_model().cluster_centers
    u2 = dc.KMeans(10, 0, init_strategy="uniform", fixed_seed=5).fit(X).fetch_model().cluster_centers
    np.testing.assert_array_equal(u1, u2)
    want = X[np.sort(np.random.RandomState(5).choice(3000, 10, replace=False))]
    np.testing.assert_array_equal(u1, want)


def test_cluster_model_transform(dc, oracle):
    rng = np.random.default_rng(3)
    X = rng.normal(size=(5000, 40)).astype(np.float32)
    C = X[rng.choice(5000, 300, replace=False)] + 0.05 * rng.normal(size=(300, 40)).astype(np.float32)
    got = dc.ClusterModel(cluster_centers=C, metric="euclidean").transform(X, n_jobs=2)
    np.testing.assert_array_equal(got, oracle.assign(X, C))
    Xr = rotated_clusters(rng, n_clusters=4, n_particles=5, per_cluster=30)
    Cr = Xr[[0, 30, 60, 90]]
    got = dc.ClusterModel(Cr, metric="minRMSD", converged=True).transform(Xr)
    np.testing.assert_array_equal(got, oracle.assign_minrmsd(Xr, Cr))


def test_minrmsd_metric_and_kmpp_binding(dc, oracle):
    # test_kmeans.py:254-265 and :267-316 with the module's own registry
    impl = dc.metrics["minRMSD"]
    rng = np.random.default_rng(4)
    x = rng.uniform(size=(1, 3 * 15)).astype(np.float32)
    y = rng.uniform(size=(1, 3 * 15)).astype(np.float32)
    assert impl.compute_metric(x, y) == float(oracle.minrmsd_rows(x, y)[0])
    assert abs(impl.compute_metric(x, y) - oracle.kabsch_rmsd_fp64(x[0], y[0])) < 2e-5 * max(
        1.0, oracle.kabsch_rmsd_fp64(x[0], y[0]))
    out = rotated_clusters(rng, n_clusters=5, n_particles=3, per_cluster=25)
    cc = impl.kmeans.init_centers_kmpp(out, k=5, random_seed=11, n_threads=1, callback=None)
    np.testing.assert_array_equal(cc, oracle.kmpp_minrmsd(out, 5, 11)[0])
    # each rotated cluster gets one label (with seed 11 every cluster holds a
    # center; some other seeds draw two centers in one cluster on this data)
    assignments = dc.ClusterModel(cc, metric="minRMSD", converged=True).transform(out)
    for i in range(5):
        assert len(np.unique(assignments[25 * i:25 * (i + 1)])) == 1
    assert impl.kmeans.init_centers_kmpp(out, k=5, random_seed=-1, n_threads=1, callback=None).shape == (5, 9)
    eu = dc.metrics["euclidean"].kmeans.init_centers_kmpp(out, 4, 9, 1, None)
    np.testing.assert_array_equal(eu, oracle.kmpp(out, 4, 9)[0])


def test_minibatch_partial_fit(dc, oracle):
    X = mixture(20000, 6, 10, 5)
    rng = np.random.default_rng(6)
    b1 = X[np.sort(rng.choice(20000, 4000, replace=False))]
    b2 = X[np.sort(rng.choice(20000, 4000, replace=False))]
    C0 = X[:15].copy()
    est = dc.MiniBatchKMeans(n_clusters=15, metric="euclidean", n_jobs=1, init_strategy="kmeans++",
                             initial_centers=C0)
    m1 = est.partial_fit(b1).fetch_model()
    r1 = oracle.lloyd(b1, C0, 1, -1.0)
    np.testing.assert_allclose(m1.cluster_centers, r1["centers"], rtol=1e-6, atol=1e-6)
    assert abs(m1.inertia - r1["inertias"][0]) <= 1e-6 * r1["inertias"][0]
    m2 = est.partial_fit(b2).fetch_model()
    r2 = oracle.lloyd(b2, m1.cluster_centers, 1, -1.0)
    np.testing.assert_allclose(m2.cluster_centers, r2["centers"], rtol=1e-6, atol=1e-6)
    assert abs(m2.inertia - r2["inertias"][0]) <= 1e-6 * r2["inertias"][0]


def test_regspace_partial_fit_over_chunks(dc, oracle):
    rng = np.random.default_rng(7)
    X = rng.uniform(-3, 3, size=(9000, 3)).astype(np.float32)
    est = dc.RegularSpace(dmin=0.7, max_centers=5000, metric="euclidean", n_jobs=1)
    for a in range(0, 9000, 2500):  # chunks, as regspace.py:146-151 feeds them
        est.partial_fit(X[a:a + 2500].astype(np.float32, order="C", copy=False), n_jobs=1)
    want, conv = oracle.regspace(X, 0.7, 5000)
    assert conv
    np.testing.assert_array_equal(est.fetch_model().cluster_centers, want)
    small = dc.RegularSpace(dmin=0.7, max_centers=40)
    with pytest.raises(Exception) as e:
        small.partial_fit(X[:3000])
        small.partial_fit(X[3000:])
    assert "MaxCentersReachedException" in e.value.__class__.__name__
    np.testing.assert_array_equal(small.fetch_model().cluster_centers, oracle.regspace(X, 0.7, 40)[0])


def test_pyemma_call_shapes_through_install(dc, oracle):
    # kmeans.py:211-262 and interface.py:164-166 verbatim in shape, through
    # `from deeptime.clustering import ...`
    assert dc.install(force=True)
    try:
        from deeptime.clustering import ClusterModel, KMeans
        X = mixture(4000, 5, 9, 8)
        estimator = KMeans(12, 40, "euclidean", tolerance=1e-5, init_strategy="kmeans++", fixed_seed=7, n_jobs=1)
        estimator.fit(X, callback_init_centers=None, callback_loop=None, n_jobs=1)
        model = estimator.fetch_model()
        ref = oracle.lloyd(X, oracle.kmpp(X, 12, 7)[0], 40, 1e-5)
        assert model.converged == ref["converged"] and len(model.inertias) == ref["n_iter"]
        dtraj = ClusterModel(cluster_centers=model.cluster_centers, metric="euclidean").transform(X)
        np.testing.assert_array_equal(dtraj, oracle.assign(X, model.cluster_centers))
    finally:
        dc.uninstall()
